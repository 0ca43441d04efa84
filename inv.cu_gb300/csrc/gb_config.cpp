// Configuration and file formats of the drop-in boundary.
//
// Config parsing keeps the reference's rules (lib/config.h:9-108): `key =
// value` lines, first token on each side, '#'-keys ignored, first definition
// wins (command line > config.ini > inherited file, one level of `inherit`),
// every value that parses completely as a float becomes f[key] and
// i[key] = round(f[key]); sources.dat / stations.dat lines are kept only when
// exactly 7 / 2 numbers parse with nothing after the last one.
#include "gb_config.h"

#include <dirent.h>
#include <stdio.h>
#include <sys/stat.h>
#include <unistd.h>

#include <cmath>
#include <cstring>
#include <fstream>
#include <sstream>

#include "gbfwi.h"

namespace gb {

static thread_local std::string g_error;
void set_error(const std::string &msg) { g_error = msg; }
const char *last_error() { return g_error.c_str(); }

static std::string strip_leading(const std::string &s) {
    size_t pos = s.find_first_not_of(" \t");
    return pos == std::string::npos ? s : s.substr(pos);
}

void Config::load_file(const std::string &file) {
    std::ifstream in(file);
    std::string line;
    while (std::getline(in, line)) {
        line = strip_leading(line);
        size_t pos = line.find('=');
        if (pos == std::string::npos) continue;
        std::istringstream ks(line.substr(0, pos)), vs(line.substr(pos + 1));
        std::string key, value;
        ks >> key;
        vs >> value;
        if (!key.empty() && !value.empty() && key[0] != '#' && raw[key].empty()) raw[key] = value;
    }
}

bool Config::parse_value(const std::string &text, float *out) {
    std::istringstream s(text);
    float v;
    s >> v;
    if (s.eof() && !s.fail()) {
        *out = v;
        return true;
    }
    return false;
}

void Config::parse() {
    f.clear();
    i.clear();
    for (auto const &kv : raw) {
        if (kv.first == "config" || kv.first == "inherit") continue;
        float v;
        if (parse_value(kv.second, &v)) {
            f[kv.first] = v;
            i[kv.first] = (int)std::round(v);
        }
    }
}

template <size_t N>
static void load_rows(const std::string &file, std::vector<std::array<float, N>> &rows) {
    std::ifstream in(file);
    std::string line;
    while (std::getline(in, line)) {
        line = strip_leading(line);
        std::istringstream s(line);
        std::array<float, N> row{};
        for (size_t q = 0; q < N; q++) s >> row[q];
        if (s.eof() && !s.fail()) rows.push_back(row);
    }
}

void Config::load_dir(const std::string &dir) {
    path = dir;
    raw["config"] = dir;
    load_file(dir + "/config.ini");
    if (!raw["inherit"].empty()) load_file(raw["inherit"]);
    parse();
    src.clear();
    rec.clear();
    load_rows<7>(dir + "/sources.dat", src);
    load_rows<2>(dir + "/stations.dat", rec);
}

float Config::fv(const std::string &k) const {
    auto it = f.find(k);
    return it == f.end() ? 0.f : it->second;
}
int Config::iv(const std::string &k) const {
    auto it = i.find(k);
    return it == i.end() ? 0 : it->second;
}
bool Config::has(const std::string &k) const { return f.count(k) != 0; }

// ------------------------------------------------------------ filesystem
void make_dirs(const std::string &p) {
    for (size_t q = 0; q < p.size(); q++)
        if (p[q] == '/' && q > 0) mkdir(p.substr(0, q).c_str(), 0777);
    mkdir(p.c_str(), 0777);
}

void clean_dir(const std::string &p) {
    DIR *d = opendir(p.c_str());
    if (!d) return;
    while (struct dirent *e = readdir(d)) {
        if (e->d_name[0] != '.') remove((p + "/" + e->d_name).c_str());
    }
    closedir(d);
    rmdir(p.c_str());
}

// ------------------------------------------------------------ .bin files
int read_bin(const std::string &file, std::vector<float> &data) {
    std::ifstream in(file, std::ios::binary);
    if (!in) {
        set_error("cannot open " + file);
        return GB_ERR_IO;
    }
    int32_t npt = 0;
    in.read(reinterpret_cast<char *>(&npt), 4);
    if (!in || npt < 0) {
        set_error("bad header in " + file);
        return GB_ERR_IO;
    }
    data.resize((size_t)npt);
    in.read(reinterpret_cast<char *>(data.data()), (std::streamsize)npt * 4);
    if (!in) {
        set_error("short file " + file);
        return GB_ERR_IO;
    }
    return GB_OK;
}

int write_bin(const std::string &file, const float *data, size_t n) {
    std::ofstream out(file, std::ios::binary);
    if (!out) {
        set_error("cannot write " + file);
        return GB_ERR_IO;
    }
    int32_t npt = (int32_t)n;
    out.write(reinterpret_cast<const char *>(&npt), 4);
    out.write(reinterpret_cast<const char *>(data), (std::streamsize)n * 4);
    return out ? GB_OK : GB_ERR_IO;
}

std::string pad6(long v) {
    std::string s = std::to_string(v);
    while (s.size() < 6) s = "0" + s;
    return s;
}

// ------------------------------------------------------------ SU traces
// Header layout written by Solver::exportTraces (solver/solver.h:38-108):
// 28 int32, 2 int16 (0, nt), 2 int16 (dt in us or 0 above 32767, 0),
// 30 float32 (index 1 = rec_x[1] - rec_x[0] when nrec > 1).
int write_su(const std::string &file, const float *traces, int nrec, int nt, float dt, float xs, float zs,
             const float *rec_x, const float *rec_z) {
    std::ofstream out(file, std::ios::binary);
    if (!out) {
        set_error("cannot write " + file);
        return GB_ERR_IO;
    }
    int32_t h1[28];
    int16_t h2[2], h3[2];
    float h4[30];
    memset(h1, 0, sizeof h1);
    memset(h4, 0, sizeof h4);
    int16_t dt_int2 = (dt * 1e6 > std::pow(2.0, 15)) ? 0 : (int16_t)(dt * 1e6);
    h1[18] = (int32_t)std::round(xs);
    h1[19] = (int32_t)std::round(zs);
    h2[0] = 0;
    h2[1] = (int16_t)nt;
    h3[0] = dt_int2;
    h3[1] = 0;
    for (int ir = 0; ir < nrec; ir++) {
        h1[0] = ir + 1;
        h1[9] = (int32_t)std::round(rec_x[ir] - xs);
        h1[20] = (int32_t)std::round(rec_x[ir]);
        h1[21] = (int32_t)std::round(rec_z[ir]);
        if (nrec > 1) h4[1] = rec_x[1] - rec_x[0];
        out.write(reinterpret_cast<const char *>(h1), sizeof h1);
        out.write(reinterpret_cast<const char *>(h2), sizeof h2);
        out.write(reinterpret_cast<const char *>(h3), sizeof h3);
        out.write(reinterpret_cast<const char *>(h4), sizeof h4);
        out.write(reinterpret_cast<const char *>(traces + (size_t)ir * nt), (std::streamsize)nt * 4);
    }
    return out ? GB_OK : GB_ERR_IO;
}

// Misfit::importTraces (misfit/misfit.h:52-90): skips each 240-byte header.
int read_su(const std::string &file, float *traces, int nrec, int nt) {
    std::ifstream in(file, std::ios::binary);
    if (!in) {
        set_error("cannot open " + file);
        return GB_ERR_IO;
    }
    for (int ir = 0; ir < nrec; ir++) {
        in.seekg(240, std::ios::cur);
        in.read(reinterpret_cast<char *>(traces + (size_t)ir * nt), (std::streamsize)nt * 4);
        if (!in) {
            set_error("short SU file " + file);
            return GB_ERR_IO;
        }
    }
    return GB_OK;
}

}  // namespace gb

// ------------------------------------------------------------ C ABI
using gb::Config;

extern "C" {

const char *gb_last_error(void) { return gb::last_error(); }
int gb_version(void) { return GB_VERSION; }

gb_config *gb_config_load(const char *dir, int nover, const char *const *overrides) {
    if (!dir) {
        gb::set_error("gb_config_load: null directory");
        return nullptr;
    }
    Config *c = new Config();
    for (int q = 0; q < nover; q++) {
        std::string a = overrides[q] ? overrides[q] : "";
        if (!a.empty() && a[0] == '-') a = a.substr(1);
        size_t pos = a.find('=');
        if (pos == std::string::npos) continue;
        c->raw[a.substr(0, pos)] = a.substr(pos + 1);
    }
    c->load_dir(dir);
    if (c->iv("clean")) gb::clean_dir(c->path + "/output");
    gb::make_dirs(c->path + "/output");
    return reinterpret_cast<gb_config *>(c);
}

gb_config *gb_config_new(const char *dir) {
    Config *c = new Config();
    c->path = dir ? dir : ".";
    c->raw["config"] = c->path;
    return reinterpret_cast<gb_config *>(c);
}

void gb_config_free(gb_config *cfg) { delete reinterpret_cast<Config *>(cfg); }

int gb_config_set(gb_config *cfg, const char *key, const char *value) {
    if (!cfg || !key || !value) return GB_ERR_ARG;
    Config *c = reinterpret_cast<Config *>(cfg);
    c->raw[key] = value;
    c->parse();
    return GB_OK;
}

int gb_config_has(const gb_config *cfg, const char *key) {
    return cfg && key && reinterpret_cast<const Config *>(cfg)->has(key);
}
float gb_config_f(const gb_config *cfg, const char *key) {
    return (cfg && key) ? reinterpret_cast<const Config *>(cfg)->fv(key) : 0.f;
}
int gb_config_i(const gb_config *cfg, const char *key) {
    return (cfg && key) ? reinterpret_cast<const Config *>(cfg)->iv(key) : 0;
}
const char *gb_config_path(const gb_config *cfg) {
    return cfg ? reinterpret_cast<const Config *>(cfg)->path.c_str() : "";
}
int gb_config_nsrc(const gb_config *cfg) { return cfg ? (int)reinterpret_cast<const Config *>(cfg)->src.size() : 0; }
int gb_config_nrec(const gb_config *cfg) { return cfg ? (int)reinterpret_cast<const Config *>(cfg)->rec.size() : 0; }

int gb_config_source(const gb_config *cfg, int is, float out[7]) {
    const Config *c = reinterpret_cast<const Config *>(cfg);
    if (!c || is < 0 || is >= (int)c->src.size() || !out) return GB_ERR_ARG;
    for (int q = 0; q < 7; q++) out[q] = c->src[is][q];
    return GB_OK;
}
int gb_config_station(const gb_config *cfg, int ir, float out[2]) {
    const Config *c = reinterpret_cast<const Config *>(cfg);
    if (!c || ir < 0 || ir >= (int)c->rec.size() || !out) return GB_ERR_ARG;
    out[0] = c->rec[ir][0];
    out[1] = c->rec[ir][1];
    return GB_OK;
}
int gb_config_add_source(gb_config *cfg, const float src[7]) {
    Config *c = reinterpret_cast<Config *>(cfg);
    if (!c || !src) return GB_ERR_ARG;
    std::array<float, 7> a;
    for (int q = 0; q < 7; q++) a[q] = src[q];
    c->src.push_back(a);
    return GB_OK;
}
int gb_config_add_station(gb_config *cfg, const float rec[2]) {
    Config *c = reinterpret_cast<Config *>(cfg);
    if (!c || !rec) return GB_ERR_ARG;
    c->rec.push_back({rec[0], rec[1]});
    return GB_OK;
}

}  // extern "C"
