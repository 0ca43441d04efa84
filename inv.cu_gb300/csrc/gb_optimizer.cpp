// Optimizer: the GB300 replacement of Optimizer (optimizer/optimizer.h),
// NLCGOptimizer (optimizer/nlcg.h) and LBFGSOptimizer (optimizer/lbfgs.h).
//
// The decision rules, restart conditions and printed lines are the
// reference's. What changes: model-vector dot products and max|.| are FP64
// reductions on the GPU (rounded to float where the line search stores them,
// as the reference's cuBLAS results are float), the quadratic fit is a small
// Householder least-squares solve in double on the host (the reference ships
// a 4x3 system to cuSOLVER), and the L-BFGS history stays in device memory
// instead of host RAM (optimizer/lbfgs.h:94-106). The line search keeps and
// computes its steps, history and slopes in float, as the reference does
// (see bracket). The L-BFGS history rotation keeps the reference's slot
// aliasing (see direction_lbfgs).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <ctime>
#include <iostream>
#include <vector>

#include "gb_solver.h"

using namespace gb;

struct gb_optimizer {
    Solver *s = nullptr;
    gb_misfit *misfit = nullptr;
    int type = 0;  // 0 NLCG, 1 L-BFGS
    bool inv[3] = {false, false, false};
    int inv_cycle = 0, inv_iteration = 0, ls_step = 0;
    float ls_step_max = 0, ls_step_init = 0, ls_thresh = 0;
    int nlcg_type = 0;
    double nlcg_thresh = 0;
    int lbfgs_mem = 0, lbfgs_used = 0;
    double lbfgs_thresh = 0;
    long eval_count = 0, inv_count = 0, ls_count = 0;
    std::vector<float> ls_lens, ls_vals, ls_gtg, ls_gtp;
    float *m_new[3] = {}, *g_new[3] = {};
    float *m_old[3] = {}, *g_old[3] = {}, *p_new[3] = {}, *p_old[3] = {};
    std::vector<std::vector<float *>> S, Y;  // [mem][3] device vectors (slots may share buffers)
    std::vector<float *> owned;             // every S/Y buffer, for release
    double *d_red = nullptr;
    double ref = 1.0;
    std::vector<double> history;
    std::vector<double> evals;  // (kind, alpha, value) per misfit evaluation
    int err = GB_OK;

    size_t n() const { return s->ncell(); }

    // ---- model-vector operations over the inverted parameters
    double dot(float *const *a, float *const *b) {
        double acc = 0.0;
        for (int ip = 0; ip < 3; ip++) {
            if (!inv[ip]) continue;
            double v = 0.0;
            if (launch_dot(a[ip], b[ip], n(), d_red, d_red + reduce_partials(), s->st) != cudaSuccess ||
                cudaMemcpyAsync(&v, d_red + reduce_partials(), 8, cudaMemcpyDeviceToHost, s->st) != cudaSuccess ||
                cudaStreamSynchronize(s->st) != cudaSuccess)
                err = GB_ERR_CUDA;
            acc += v;
        }
        return acc;
    }
    double amax(float *const *a) {
        double m = 0.0;
        for (int ip = 0; ip < 3; ip++) {
            if (!inv[ip]) continue;
            double v = 0.0;
            if (launch_amax(a[ip], n(), d_red, d_red + reduce_partials(), s->st) != cudaSuccess ||
                cudaMemcpyAsync(&v, d_red + reduce_partials(), 8, cudaMemcpyDeviceToHost, s->st) != cudaSuccess ||
                cudaStreamSynchronize(s->st) != cudaSuccess)
                err = GB_ERR_CUDA;
            m = std::max(m, v);
        }
        return m;
    }
    // c = ka*a + kb*b (b may be null), float coefficients as in device::calc
    void calc(float *const *c, double ka, float *const *a, double kb = 0, float *const *b = nullptr) {
        for (int ip = 0; ip < 3; ip++) {
            if (!inv[ip]) continue;
            if (launch_axpby(c[ip], (float)ka, a[ip], (float)kb, b ? b[ip] : nullptr, n(), s->st) != cudaSuccess)
                err = GB_ERR_CUDA;
        }
    }
    void copy(float *const *d, float *const *src) {
        for (int ip = 0; ip < 3; ip++)
            if (inv[ip] && cudaMemcpyAsync(d[ip], src[ip], n() * 4, cudaMemcpyDeviceToDevice, s->st) != cudaSuccess)
                err = GB_ERR_CUDA;
    }
    double angle(float *const *p, float *const *g, double k = 1) {
        const double xx = dot(p, p), yy = dot(g, g), xy = k * dot(p, g);
        return std::acos(xy / std::sqrt(xx * yy));
    }

    // kind: 1 gradient (start of an iteration), 0 line-search step, 2 final;
    // alpha: the step the line search took to this model (0 otherwise)
    double evaluate(bool kernel, int kind, double alpha) {
        double v = 0.0;
        int rc = gb_misfit_run(misfit, kernel, 0, &v);
        if (rc) err = rc;
        evals.insert(evals.end(), {(double)kind, alpha, v});
        return v;
    }

    // ---- line search (optimizer/optimizer.h:151-357), in float like the
    // reference's: a rule that took its decisions in double would part from
    // the reference's on the same history, and not only by chance: after the
    // first step is clamped to 0.618034 * step_max, the golden-ratio
    // extrapolation 1.618034 * x lands within one float ulp of step_max, and
    // whether it exceeds step_max decides between evaluating there (status 0)
    // and accepting it unevaluated (status 1).
    // Least-squares quadratic p0 x^2 + p1 x + p2 through n points (double).
    static void polyfit(const double *x, const double *y, double *p, int n) {
        double A[4][3], b[4];
        for (int i = 0; i < n; i++) {
            A[i][0] = x[i] * x[i];
            A[i][1] = x[i];
            A[i][2] = 1;
            b[i] = y[i];
        }
        const int nc = 3;
        for (int k = 0; k < nc && k < n; k++) {
            double norm = 0;
            for (int i = k; i < n; i++) norm += A[i][k] * A[i][k];
            norm = std::sqrt(norm);
            if (norm == 0) continue;
            const double alpha = A[k][k] > 0 ? -norm : norm;
            double v[4] = {0, 0, 0, 0};
            for (int i = k; i < n; i++) v[i] = A[i][k];
            v[k] -= alpha;
            double vv = 0;
            for (int i = k; i < n; i++) vv += v[i] * v[i];
            if (vv == 0) continue;
            for (int j = k; j < nc; j++) {
                double d = 0;
                for (int i = k; i < n; i++) d += v[i] * A[i][j];
                for (int i = k; i < n; i++) A[i][j] -= 2 * d / vv * v[i];
            }
            double d = 0;
            for (int i = k; i < n; i++) d += v[i] * b[i];
            for (int i = k; i < n; i++) b[i] -= 2 * d / vv * v[i];
        }
        for (int k = std::min(nc, n) - 1; k >= 0; k--) {
            double acc = b[k];
            for (int j = k + 1; j < nc; j++) acc -= A[k][j] * p[j];
            p[k] = A[k][k] != 0 ? acc / A[k][k] : 0;
        }
        for (int k = std::min(nc, n); k < nc; k++) p[k] = 0;
    }

    int history_of(int step_count, std::vector<float> &x, std::vector<float> &f) {
        x.resize(step_count + 1);
        f.resize(step_count + 1);
        for (int i = 0; i < step_count + 1; i++) {
            const long j = ls_count - 1 - step_count + i;
            x[i] = ls_lens[j];
            f[i] = ls_vals[j];
        }
        for (int i = 0; i < step_count + 1; i++)
            for (int j = i + 1; j < step_count + 1; j++)
                if (x[j] < x[i]) {
                    std::swap(x[i], x[j]);
                    std::swap(f[i], f[j]);
                }
        int update_count = 0;
        for (long i = 0; i < ls_count; i++)
            if (std::fabs(ls_lens[i]) < 1e-6) update_count++;
        if (update_count > 0) update_count--;
        return update_count;
    }
    static int argmin(const float *f, int n) {
        float m = f[0];
        int idx = 0;
        for (int i = 1; i < n; i++)
            if (f[i] < m) {
                m = f[i];
                idx = i;
            }
        return idx;
    }
    static bool check_bracket(const float *f, int n) {
        const int imin = argmin(f, n);
        const float fmin = f[imin];
        if (fmin < f[0])
            for (int i = imin; i < n; i++)
                if (f[i] > fmin) return true;
        return false;
    }
    bool good_enough(const float *x, const float *f, int n, float &x0) {
        const float thresh = std::log10(ls_thresh);
        if (!check_bracket(f, n)) return false;
        const int idx = argmin(f, n) - 1;
        const int fitlen = std::min(4, n - idx);
        double xd[4], fd[4], p[3];
        for (int i = 0; i < fitlen; i++) {
            xd[i] = x[idx + i];
            fd[i] = f[idx + i];
        }
        polyfit(xd, fd, p, fitlen);
        const float p0 = (float)p[0], p1 = (float)p[1];  // optimizer.h:174-177
        if (p0 > 0) {
            x0 = -p1 / (2 * p0);
        } else if (p[0] > 0) {
            // The float coefficient underflowed (steps of ~1e20: a model of
            // ~1e10 over gradients of ~1e-10): the reference then prints "line
            // search error" and leaves bracket's step uninitialised. The
            // double fit's minimum is taken instead.
            x0 = (float)(-p[1] / (2 * p[0]));
        } else {
            // No positive curvature: the reference's step is uninitialised
            // here too. The search ends at the best point evaluated, so that
            // it cannot re-evaluate that point forever.
            std::cout << "  line search error" << std::endl;
            x0 = x[argmin(f, n)];
            return true;
        }
        for (int i = 1; i < n; i++)
            if (std::fabs(std::log10(x[i] / x0)) < thresh) return true;
        return false;
    }
    static float backtrack2(float f0, float g0, float x1, float f1, float b1, float b2) {
        float x2 = -g0 * x1 * x1 / (2 * (f1 - f0 - g0 * x1));
        if (x2 > b2 * x1)
            x2 = b2 * x1;
        else if (x2 < b1 * x1)
            x2 = b1 * x1;
        return x2;
    }
    float bracket(int step_count, float step_max, int &status) {
        std::vector<float> x, f;
        float alpha = 0;
        const int update_count = history_of(step_count, x, f);
        if (step_count == 0) {
            if (update_count == 0) {
                alpha = 1 / ls_gtg[inv_count - 1];
                status = 0;
            } else {
                const int idx = argmin(ls_vals.data(), (int)ls_count - 1);
                alpha = ls_lens[idx] * ls_gtp[inv_count - 2] / ls_gtp[inv_count - 1];
                status = 0;
            }
        } else if (check_bracket(f.data(), step_count + 1)) {
            if (good_enough(x.data(), f.data(), step_count + 1, alpha)) {
                alpha = x[argmin(f.data(), step_count + 1)];
                status = 1;
            } else {
                status = 0;
            }
        } else if (step_count <= ls_step) {
            int i;
            for (i = 1; i < step_count + 1; i++)
                if (f[i] > f[0]) break;
            if (i == step_count + 1) {
                alpha = 1.618034 * x[step_count];
                status = 0;
            } else {
                const float slope = ls_gtp[inv_count - 1] / ls_gtg[inv_count - 1];
                alpha = backtrack2(f[0], slope, x[1], f[1], 0.1f, 0.5f);
                status = 0;
            }
        } else {
            alpha = 0;
            status = -1;
        }
        if (alpha > step_max) {
            if (step_count == 0) {
                alpha = 0.618034 * step_max;
                status = 0;
            } else {
                alpha = step_max;
                status = 1;
            }
        }
        return alpha;
    }
    float backtrack(int step_count, float step_max, int &status) {
        std::vector<float> x, f;
        const int update_count = history_of(step_count, x, f);
        const int idx = argmin(f.data(), step_count + 1);
        float alpha;
        if (update_count == 0) {
            alpha = bracket(step_count, step_max, status);
        } else if (step_count == 0) {
            alpha = std::min(1.0f, step_max);
            status = 0;
        } else if (f[idx] < f[0]) {
            alpha = x[idx];
            status = 1;
        } else if (step_count <= ls_step) {
            const float slope = ls_gtp[inv_count - 1] / ls_gtg[inv_count - 1];
            alpha = backtrack2(f[0], slope, x[1], f[1], 0.1f, 0.5f);
            status = 0;
        } else {
            alpha = 0;
            status = -1;
        }
        return alpha;
    }
    float calc_step(int step_count, float step_max, int &status) {
        return type == 0 ? bracket(step_count, step_max, status) : backtrack(step_count, step_max, status);
    }
    long ls_cap() const { return std::max(1L, (long)inv_iteration * ls_step); }
    void push_ls(float len, float val) {
        if ((size_t)ls_count >= ls_lens.size()) {
            ls_lens.resize(ls_count + 1);
            ls_vals.resize(ls_count + 1);
        }
        ls_lens[ls_count] = len;
        ls_vals[ls_count] = val;
        ls_count++;
    }
    void restart_search() {
        calc(p_new, -1, g_new);
        ls_count = 0;
        inv_count = 1;
        if (type == 1) lbfgs_used = 0;
    }

    // Optimizer::lineSearch (optimizer/optimizer.h:360-419)
    // f: the misfit, a float in the reference (misfit->run)
    int line_search(double f_run) {
        const float f = (float)f_run;
        int status = 0;
        float alpha = 0;
        const float norm_m = (float)amax(m_new), norm_p = (float)amax(p_new);
        const float gtg = (float)dot(g_new, g_new), gtp = (float)dot(g_new, p_new);
        const float step_max = ls_step_max * norm_m / norm_p;
        int step_count = 0;
        push_ls(0, f);
        if ((size_t)inv_count > ls_gtg.size()) {
            ls_gtg.resize(inv_count);
            ls_gtp.resize(inv_count);
        }
        ls_gtg[inv_count - 1] = gtg;
        ls_gtp[inv_count - 1] = gtp;
        float alpha_current = 0;
        if (ls_step_init != 0 && ls_count <= 1)
            alpha = ls_step_init * norm_m / norm_p;
        else
            alpha = calc_step(step_count, step_max, status);
        while (true) {
            // The reference keeps inv_iteration * ls_step steps
            // (optimizer.h:485-487) and writes past them after that; here a
            // search that has used them all fails as one past ls_step does.
            if (ls_count >= ls_cap()) status = -1;
            if (status >= 0) {
                calc(m_new, 1, m_new, alpha - alpha_current, p_new);
                alpha_current = alpha;
                const double v = evaluate(false, 0, alpha);
                if (err) return -1;
                push_ls(alpha, (float)v);
                eval_count++;
                step_count++;
                alpha = calc_step(step_count, step_max, status);
                std::cout << "  step " << (step_count < 10 ? "0" : "") << step_count
                          << "  misfit = " << ls_vals[ls_count - 1] / (float)ref << std::endl;
            }
            if (status > 0) {
                std::cout << "  alpha = " << alpha << std::endl;
                calc(m_new, 1, m_new, alpha - alpha_current, p_new);
                return status;
            } else if (status < 0) {
                calc(m_new, 1, m_new, -alpha_current, p_new);
                if (angle(p_new, g_new, -1) < 1e-3) {
                    std::cout << "  line search failed" << std::endl;
                    return status;
                }
                std::cout << "  restarting line search..." << std::endl;
                restart_search();
                return line_search(f_run);
            }
        }
    }

    // NLCGOptimizer::computeDirection (optimizer/nlcg.h:24-52)
    int direction_nlcg() {
        inv_count++;
        if (inv_count == 1) {
            calc(p_new, -1, g_new);
            return 0;
        }
        if (inv_cycle && inv_cycle < inv_count) {
            std::cout << "  restarting NLCG... [periodic restart]" << std::endl;
            return -1;
        }
        double beta = 0;
        if (nlcg_type == 0) {
            beta = dot(g_new, g_new) / dot(g_old, g_old);
        } else if (nlcg_type == 1) {
            calc(p_new, 1, g_new, -1, g_old);
            beta = dot(g_new, p_new) / dot(g_old, g_old);
        }
        calc(p_new, -1, g_new, beta, p_old);
        if (angle(g_new, g_old) < nlcg_thresh) {
            std::cout << "  restarting NLCG... [loss of conjugacy]" << std::endl;
            return -1;
        }
        if (dot(p_new, g_new) > 0) {
            std::cout << "  restarting NLCG... [not a descent direction]" << std::endl;
            return -1;
        }
        return 1;
    }

    // LBFGSOptimizer::computeDirection (optimizer/lbfgs.h:18-91)
    int direction_lbfgs() {
        inv_count++;
        if (inv_count == 1) {
            calc(p_new, -1, g_new);
            return 0;
        }
        if (inv_cycle && inv_cycle < inv_count) {
            std::cout << "  restarting LBFGS... [periodic restart]" << std::endl;
            return -1;
        }
        // lbfgs.h:29-36 binds a reference to the last slot, shifts the slots
        // up by one (overwriting the last with its predecessor) and then puts
        // what the reference now names into slot 0: after the rotation slot 0
        // and slot mem-1 share one buffer, so once the memory is full the
        // newest pair also stands in the oldest pair's place. Kept as is.
        const int mem = (int)S.size();
        for (int i = mem - 1; i > 0; i--) {
            S[i] = S[i - 1];
            Y[i] = Y[i - 1];
        }
        S[0] = S[mem - 1];
        Y[0] = Y[mem - 1];
        calc(S[0].data(), 1, m_new, -1, m_old);
        calc(Y[0].data(), 1, g_new, -1, g_old);
        if (lbfgs_used < lbfgs_mem) lbfgs_used++;
        std::vector<double> rh(lbfgs_used), al(lbfgs_used);
        copy(p_new, g_new);
        double sty = 1, yty = 1;
        for (int i = 0; i < lbfgs_used; i++) {
            rh[i] = 1 / dot(Y[i].data(), S[i].data());
            al[i] = rh[i] * dot(S[i].data(), p_new);
            calc(p_new, 1, p_new, -al[i], Y[i].data());
            if (i == 0) {
                sty = 1 / rh[i];
                yty = dot(Y[i].data(), Y[i].data());
            }
        }
        calc(p_new, sty / yty, p_new);
        for (int i = lbfgs_used - 1; i >= 0; i--) {
            const double be = rh[i] * dot(Y[i].data(), p_new);
            calc(p_new, 1, p_new, al[i] - be, S[i].data());
        }
        const double pi = 3.1415927f;
        const double a = angle(g_new, p_new);
        if (a >= pi / 2) {
            std::cout << "  restarting LBFGS... [not a descent direction]" << std::endl;
            return -1;
        } else if (a > pi / 2 - lbfgs_thresh) {
            std::cout << "  restarting LBFGS... [practical safeguard]" << std::endl;
            return -1;
        }
        calc(p_new, -1, p_new);
        return 1;
    }

    // Optimizer::run (optimizer/optimizer.h:428-467)
    int run() {
        int rc = gb_export_axis(reinterpret_cast<gb_solver *>(s));
        if (!rc) rc = gb_export_model(reinterpret_cast<gb_solver *>(s), 0);
        if (rc) return rc;
        history.clear();
        evals.clear();
        const clock_t t0 = clock();
        for (int iter = 0; iter < inv_iteration; iter++) {
            std::cout << "\nStarting iteration " << iter + 1 << " / " << inv_iteration << std::endl;
            const double f = evaluate(true, 1, 0.0);
            if (err) return err;
            if (iter == 0) ref = f;
            eval_count += 2;
            std::cout << "  step 00  misfit = " << (float)(f / ref) << std::endl;
            history.push_back(f);
            if ((type == 0 ? direction_nlcg() : direction_lbfgs()) < 0) restart_search();
            copy(m_old, m_new);
            copy(p_old, p_new);
            copy(g_old, g_new);
            if (err) return err;
            if (line_search(f) < 0) {
                if (err) return err;
                break;
            }
            rc = gb_export_kernel(reinterpret_cast<gb_solver *>(s), iter + 1);
            if (!rc) rc = gb_export_model(reinterpret_cast<gb_solver *>(s), iter + 1);
            if (rc) return rc;
        }
        const float elapsed = (float)(clock() - t0) / CLOCKS_PER_SEC;
        const double final_f = evaluate(false, 2, 0.0);
        if (err) return err;
        history.push_back(final_f);
        std::cout << "\nFinal misfit: " << (float)(final_f / ref) << std::endl;
        std::cout << "Elapsed time: ";
        if (elapsed > 60) {
            const size_t t_min = (size_t)(elapsed / 60);
            const size_t t_sec = (size_t)(elapsed - t_min * 60);
            std::cout << t_min << "min " << t_sec << "s" << std::endl;
        } else {
            std::cout << std::round(elapsed) << std::endl;
        }
        return GB_OK;
    }
};

extern "C" {

gb_optimizer *gb_optimizer_create(const gb_config *cfg, gb_solver *sol, gb_misfit *m) {
    if (!cfg || !sol || !m) {
        set_error("gb_optimizer_create: null argument");
        return nullptr;
    }
    const Config &c = *reinterpret_cast<const Config *>(cfg);
    Solver &s = sol->s;
    if (!s.adj) {
        set_error("gb_optimizer_create: the solver has no kernels (mode must be 0 or 2)");
        return nullptr;
    }
    gb_optimizer *o = new gb_optimizer();
    o->s = &s;
    o->misfit = m;
    o->type = c.iv("optimizer");
    if (o->type != 0 && o->type != 1) {
        set_error("gb_optimizer_create: optimizer must be 0 (NLCG) or 1 (L-BFGS)");
        delete o;
        return nullptr;
    }
    o->inv[0] = s.inv_lambda;
    o->inv[1] = s.inv_mu;
    o->inv[2] = s.inv_rho;
    o->inv_iteration = c.iv("inv_iteration");
    o->inv_cycle = c.iv("inv_cycle");
    o->ls_step = c.iv("ls_step");
    o->ls_step_max = (float)c.fv("ls_step_max");
    o->ls_step_init = (float)c.fv("ls_step_init");
    o->ls_thresh = (float)c.fv("ls_thresh");
    o->nlcg_type = c.iv("nlcg_type");
    o->nlcg_thresh = c.fv("nlcg_thresh");
    o->lbfgs_mem = c.iv("lbfgs_mem");
    o->lbfgs_thresh = c.fv("lbfgs_thresh");
    if (o->type == 1 && o->lbfgs_mem < 1) {
        // the reference indexes lbfgs_S[lbfgs_mem - 1] (optimizer/lbfgs.h:29)
        set_error("gb_optimizer_create: lbfgs_mem must be at least 1 for L-BFGS");
        delete o;
        return nullptr;
    }
    o->ls_lens.resize(std::max(1, o->inv_iteration * o->ls_step));
    o->ls_vals.resize(o->ls_lens.size());
    o->ls_gtg.resize(std::max(1, o->inv_iteration));
    o->ls_gtp.resize(o->ls_gtg.size());
    o->m_new[0] = s.lambda;
    o->m_new[1] = s.mu;
    o->m_new[2] = s.rho;
    o->g_new[0] = s.k_lambda;
    o->g_new[1] = s.k_mu;
    o->g_new[2] = s.k_rho;
    const size_t bytes = s.ncell() * 4;
    bool ok = cudaMalloc(&o->d_red, (reduce_partials() + 1) * sizeof(double)) == cudaSuccess;
    for (int ip = 0; ip < 3 && ok; ip++)
        for (float **v : {&o->m_old[ip], &o->g_old[ip], &o->p_new[ip], &o->p_old[ip]})
            ok = ok && cudaMalloc(v, bytes) == cudaSuccess && cudaMemset(*v, 0, bytes) == cudaSuccess;
    if (o->type == 1) {
        o->S.assign(std::max(o->lbfgs_mem, 1), std::vector<float *>(3, nullptr));
        o->Y.assign(std::max(o->lbfgs_mem, 1), std::vector<float *>(3, nullptr));
        for (int q = 0; q < o->lbfgs_mem && ok; q++)
            for (int ip = 0; ip < 3 && ok; ip++)
                if (o->inv[ip]) {
                    ok = cudaMalloc(&o->S[q][ip], bytes) == cudaSuccess;
                    if (ok) o->owned.push_back(o->S[q][ip]);
                    ok = ok && cudaMalloc(&o->Y[q][ip], bytes) == cudaSuccess;
                    if (ok) o->owned.push_back(o->Y[q][ip]);
                }
    }
    if (!ok) {
        set_error("gb_optimizer_create: device allocation failed");
        gb_optimizer_destroy(o);
        return nullptr;
    }
    return o;
}

int gb_optimizer_run(gb_optimizer *o) {
    if (!o) return GB_ERR_ARG;
    o->err = GB_OK;
    int rc = o->run();
    return rc ? rc : o->err;
}

int gb_optimizer_history(gb_optimizer *o, double *out, int n) {
    if (!o) return 0;
    const int k = std::min<int>(n, (int)o->history.size());
    for (int i = 0; i < k && out; i++) out[i] = o->history[i];
    return (int)o->history.size();
}

double gb_linesearch_step(int optimizer, const double *lens, const double *vals, int ls_count, const double *gtg,
                          const double *gtp, int inv_count, int step_count, int ls_step, double ls_thresh,
                          double step_max, int *status) {
    if (status) *status = -2;
    if ((optimizer != 0 && optimizer != 1) || !lens || !vals || !gtg || !gtp || !status || step_count < 0 ||
        ls_count < step_count + 1 || inv_count < 1 || !(ls_thresh > 1)) {
        set_error("gb_linesearch_step: invalid history");
        return 0;
    }
    gb_optimizer o;  // host state only: the step rule touches no device memory
    o.type = optimizer;
    o.ls_step = ls_step;
    o.ls_thresh = (float)ls_thresh;
    o.ls_lens.assign(lens, lens + ls_count);
    o.ls_vals.assign(vals, vals + ls_count);
    o.ls_count = ls_count;
    o.ls_gtg.assign(gtg, gtg + inv_count);
    o.ls_gtp.assign(gtp, gtp + inv_count);
    o.inv_count = inv_count;
    std::vector<float> x, f;
    if (step_count == 0 && o.history_of(0, x, f) > 0 && inv_count < 2) {
        // the rule then scales the previous iteration's step (optimizer.h:275-277)
        set_error("gb_linesearch_step: an earlier iteration in the history needs inv_count >= 2");
        return 0;
    }
    int st = 0;
    const float a = o.calc_step(step_count, (float)step_max, st);
    *status = st;
    return a;
}

int gb_optimizer_evaluations(gb_optimizer *o, double *out, int n) {
    if (!o) return 0;
    const int cnt = (int)(o->evals.size() / 3);
    const int k = std::min(n, cnt);
    for (int i = 0; i < 3 * k && out; i++) out[i] = o->evals[i];
    return cnt;
}

void gb_optimizer_destroy(gb_optimizer *o) {
    if (!o) return;
    // the solver may already be destroyed: wait for the device instead of its stream
    cudaDeviceSynchronize();
    for (int ip = 0; ip < 3; ip++)
        for (float *v : {o->m_old[ip], o->g_old[ip], o->p_new[ip], o->p_old[ip]}) cudaFree(v);
    for (float *p : o->owned) cudaFree(p);
    cudaFree(o->d_red);
    delete o;
}

}  // extern "C"
