// Host-side configuration object and file helpers (see gb_config.cpp).
#pragma once

#include <array>
#include <map>
#include <string>
#include <vector>

namespace gb {

// Mirror of the reference's Config (lib/config.h:86-108).
struct Config {
    std::string path;
    std::map<std::string, std::string> raw;
    std::map<std::string, float> f;
    std::map<std::string, int> i;
    std::vector<std::array<float, 7>> src;  // x z type f0 t0 angle amp
    std::vector<std::array<float, 2>> rec;  // x z

    void load_file(const std::string &file);
    void load_dir(const std::string &dir);
    void parse();
    static bool parse_value(const std::string &text, float *out);
    float fv(const std::string &k) const;
    int iv(const std::string &k) const;
    bool has(const std::string &k) const;
};

void make_dirs(const std::string &p);
void clean_dir(const std::string &p);
int read_bin(const std::string &file, std::vector<float> &data);
int write_bin(const std::string &file, const float *data, size_t n);
std::string pad6(long v);
int write_su(const std::string &file, const float *traces, int nrec, int nt, float dt, float xs, float zs,
             const float *rec_x, const float *rec_z);
int read_su(const std::string &file, float *traces, int nrec, int nt);

}  // namespace gb
