// tm_sweep -- command-line sweep driver over libtm.so.
//
// Keeps the reference drivers' positional arguments
//   dt t_max L r a_start a_end div dP PREFIX
// (simulations/Percolation_FD/order_1stocDP.cpp:122-133,
//  simulations/Rietkerk_FPE/order_1stoc_test_rietkerk.cpp:99-110) and the
// sweep of critical_exp_delta (stochasticSPDP.cpp:1309-1422): div values of a
// (linspace a_start..a_end), r replicates each, measurements every step while
// t <= 1 and at logarithm10_time_bins(t_max, dt).  All div x r instances run as
// one GPU batch instead of one OpenMP thread per a.
//
// Options (after the positional arguments):
//   --model dp|multisp|rietkerk   classic DP (Euler-exact remainder, exact sampler),
//                                 MultiSp DP (RK4, Gaussian above 100, clamp 1e-12),
//                                 Rietkerk P,W,O (a = rainfall R)
//   --precision fp64|fp32  --b B --D D --sigma S --dx DX --seed N --out DIR --device K
// Initial frame: rho = 1 + dP everywhere (init_fullframe + kick); Rietkerk
// P = 1 + dP, W = 0.5, O = 1.
// Output (DIR, default "."), numbers formatted as the reference prints them:
//   TimeSeries/PRELIM_AGG_<PREFIX>_G_<L>_T_<tmax>_dt_<dt>_a_<a>_R_<r>.csv   per a
//   FRAME_<PREFIX>_G_<L>_T_<tmax>_dt_<dt>_a_<a>_R_0.csv                  final frame, replicate 0
//   <PREFIX>_P_c_Delta_G_<L>_T_<tmax>_dt_<dt>_a1_<a_start>_a2_<a_end>_R_<r>.csv   sweep table
// Exit status 0 on success, 1 on bad arguments, 2 on a library error.
#include "../../include/tm.h"

#include <sys/stat.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

namespace {

std::string num(double v)
{
    std::ostringstream o;
    o << v;
    return o.str();
}

// measurement times: 10^0 .. 10^floor1(log10 t_max), 25 per decade, on the dt grid
std::vector<double> log10_time_bins(double t_max, double dt)
{
    std::vector<double> out;
    if (t_max <= 1) return out;
    const double tend = std::floor(std::log10(t_max) * 10.) / 10.0;
    for (double p = 0.0; p <= tend; p += 0.04) {
        double t = static_cast<int>(std::pow(10, p) / dt) * dt;
        if (t <= 1.0) t = t + dt;
        if (out.empty() || t != out.back()) out.push_back(t);
    }
    for (int i = (int)out.size() - 1; i > 0; --i)
        if (out[i] < out[i - 1] + dt / 2.0) out.erase(out.begin() + i);
    return out;
}

int fail(const char* what, int rc)
{
    std::fprintf(stderr, "tm_sweep: %s: %s\n", what, tm_error_string(rc));
    return 2;
}

}  // namespace

int main(int argc, char** argv)
{
    if (argc < 10) {
        std::fprintf(stderr, "usage: tm_sweep dt t_max L r a_start a_end div dP PREFIX [--model dp|multisp|rietkerk] "
                             "[--precision fp64|fp32] [--b B] [--D D] [--sigma S] [--dx DX] [--seed N] [--out DIR]\n");
        return 1;
    }
    const double dt = std::atof(argv[1]), t_max = std::atof(argv[2]);
    const int L = std::atoi(argv[3]), r = std::atoi(argv[4]);
    const double a_st = std::atof(argv[5]), a_end = std::atof(argv[6]);
    const int div = std::atoi(argv[7]);
    const double dP = std::atof(argv[8]);
    const std::string prefix = argv[9];
    std::string model = "dp", out = ".";
    int precision = TM_FP64, device = 0;
    double b = 2.0, D = 1.0, sigma = 1.0, dx = 1.0;
    unsigned long long seed = 0;
    for (int i = 10; i + 1 < argc; i += 2) {
        const std::string k = argv[i], v = argv[i + 1];
        if (k == "--model") model = v;
        else if (k == "--precision") precision = (v == "fp32") ? TM_FP32 : TM_FP64;
        else if (k == "--b") b = std::atof(v.c_str());
        else if (k == "--D") D = std::atof(v.c_str());
        else if (k == "--sigma") sigma = std::atof(v.c_str());
        else if (k == "--dx") dx = std::atof(v.c_str());
        else if (k == "--seed") seed = std::strtoull(v.c_str(), nullptr, 10);
        else if (k == "--out") out = v;
        else if (k == "--device") device = std::atoi(v.c_str());
        else { std::fprintf(stderr, "tm_sweep: unknown option %s\n", k.c_str()); return 1; }
    }
    if (!(dt > 0) || !(t_max > 1) || L < 1 || r < 1 || div < 1 ||
        (model != "dp" && model != "multisp" && model != "rietkerk")) {
        std::fprintf(stderr, "tm_sweep: invalid arguments\n");
        return 1;
    }
    const bool rk = model == "rietkerk";
    // a values (linspace, stochasticSPDP.cpp:254-279)
    std::vector<double> av;
    if (div == 1) av.push_back(a_st);
    else {
        const double delta = (a_end - a_st) / (div - 1);
        for (int i = 0; i < div - 1; ++i) av.push_back(a_st + delta * i);
        av.push_back(a_end);
    }
    // measurement steps: every step while t <= 1, then the log-spaced times
    std::vector<double> times;
    for (double t = 0; t <= 1; t += dt) times.push_back(t);
    const int n_early = (int)times.size();
    for (double t : log10_time_bins(t_max, dt)) times.push_back(t);
    std::vector<int64_t> steps;
    for (double t : times) steps.push_back((int64_t)std::llround(t / dt));
    const int n_meas = (int)steps.size();
    const int64_t n_steps = steps.back();

    const int n_inst = div * r;
    std::vector<tm_instance> inst(n_inst);
    for (int ia = 0; ia < div; ++ia)
        for (int j = 0; j < r; ++j) inst[ia * r + j] = tm_instance{L, 0, seed + (unsigned long long)(ia * r + j), av[ia], 0.0};
    const int nf = rk ? 3 : 1;
    std::vector<int64_t> off(n_inst), fs(n_inst);
    const int64_t total = tm_layout(inst.data(), n_inst, nf, off.data(), fs.data());
    const size_t es = precision == TM_FP64 ? 8 : 4;
    std::vector<unsigned char> init((size_t)total * es, 0);
    for (int k = 0; k < n_inst; ++k)
        for (int f = 0; f < nf; ++f) {
            const double v = rk ? (f == 0 ? 1.0 + dP : (f == 1 ? 0.5 : 1.0)) : 1.0 + dP;
            for (int64_t i = 0; i < (int64_t)L * L; ++i) {
                const size_t at = (size_t)(off[k] + f * fs[k] + i) * es;
                if (es == 8) std::memcpy(&init[at], &v, 8);
                else { const float fv = (float)v; std::memcpy(&init[at], &fv, 4); }
            }
        }

    tm_ctx* ctx = nullptr;
    int rc = tm_create(&ctx, device);
    if (rc) return fail("tm_create", rc);
    const int W = rk ? 4 : 2;
    std::vector<double> obs((size_t)n_meas * n_inst * W);
    std::vector<uint32_t> status(n_inst);
    std::vector<unsigned char> fin((size_t)total * es);
    if (rk) {
        tm_rietkerk_model m = {0.2, 5.0, 0.2, 0.05, 5.0, 10.0, 0.25, 0.2, 0.1, 0.1, 100.0, sigma, dt, dx, 0.0, 1e-10,
                               TM_SAMPLER_REF_GAUSS100, 0};
        rc = tm_run_rietkerk(ctx, &m, inst.data(), n_inst, precision, init.data(), n_steps, steps.data(), n_meas,
                             obs.data(), status.data(), fin.data());
    } else {
        tm_dp_model m = {b, 0.0, D, sigma, dt, dx, 0.0, 0.0, TM_REM_EULER_EXACT, TM_SAMPLER_EXACT, 0, 5, 1, 0};
        if (model == "multisp") {
            m.remainder = TM_REM_RK4; m.sampler = TM_SAMPLER_REF_GAUSS100;
            m.clamp_lo = -1e-80; m.clamp_eps = 1e-12;
        }
        rc = tm_run_dp(ctx, &m, inst.data(), n_inst, precision, init.data(), n_steps, steps.data(), n_meas,
                       obs.data(), status.data(), fin.data());
    }
    tm_destroy(ctx);
    if (rc) return fail("run", rc);

    mkdir(out.c_str(), 0755);
    mkdir((out + "/TimeSeries").c_str(), 0755);
    const std::string tag = "_G_" + num(L) + "_T_" + num(t_max) + "_dt_" + num(dt);
    std::ofstream stats(out + "/" + prefix + "_P_c_Delta" + tag + "_a1_" + num(a_st) + "_a2_" + num(a_end) + "_R_" +
                        num(r) + ".csv");
    stats << " a , L, t ,  <<Rho(x; t)>_x>_r, Var[<Rho(t)>_x]_r, # Surviving Runs, # Active Sites, # Surviving Runs Alt \n";
    for (int ia = 0; ia < div; ++ia) {
        std::ostringstream prelim;
        prelim << " a , r, L, t , <<P(x; t)>_x>_r, Var[<P(x; t)>_x]_r, # Surviving Runs P(x; t), # Active Sites P(x; t), \n";
        for (int i = 0; i < n_meas; ++i) {
            // statistics over the replicates still active at this time
            double s = 0, s2 = 0, act = 0;
            int ns = 0;
            for (int j = 0; j < r; ++j) {
                const double* o = &obs[((size_t)i * n_inst + ia * r + j) * W];
                const double mean = o[0], active = o[W - 1];
                if (active > 0) { ++ns; s += mean; s2 += mean * mean; act += active; }
            }
            const double mu = ns ? s / ns : 0.0;
            const double var = ns > 1 ? (s2 - ns * mu * mu) / (ns - 1) : 0.0;
            const double am = ns ? act / ns : 0.0;
            const double alt = i < n_early ? (double)r : (double)ns;
            stats << av[ia] << "," << L << "," << times[i] << "," << mu << "," << var << "," << ns << "," << am << ","
                  << alt << "\n";
            prelim << av[ia] << "," << r << "," << L << "," << times[i] << "," << mu << "," << var << "," << ns << ","
                   << am << ",\n";
        }
        std::ofstream pf(out + "/TimeSeries/PRELIM_AGG_" + prefix + tag + "_a_" + num(av[ia]) + "_R_" + num(r) + ".csv");
        pf << prelim.str();
        // final frame of replicate 0 (save_frame format)
        std::ofstream ff(out + "/FRAME_" + prefix + tag + "_a_" + num(av[ia]) + "_R_0.csv");
        ff << (rk ? "a_c,  x,  P(x; t), W(x; t), O(x; t) \n" : "a_c,  x,  P(x; t) \n");
        const int k = ia * r;
        for (int64_t i = 0; i < (int64_t)L * L; ++i) {
            ff << av[ia] << "," << i;
            for (int f = 0; f < nf; ++f) {
                const size_t at = (size_t)(off[k] + f * fs[k] + i) * es;
                double v;
                if (es == 8) std::memcpy(&v, &fin[at], 8);
                else { float fv; std::memcpy(&fv, &fin[at], 4); v = fv; }
                ff << "," << v;
            }
            ff << "\n";
        }
    }
    unsigned int any = 0;
    for (auto x : status) any |= x;
    if (any) std::fprintf(stderr, "tm_sweep: status bits 0x%x (nan=1, negative=2, sampler cap=4)\n", any);
    return 0;
}
