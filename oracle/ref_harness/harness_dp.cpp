// C-callable harness around the reference's own DP functions
// (simulations/Percolation_FD/stochasticSPDP.cpp), compiled from the reference
// sources by oracle/Makefile.  TEST INFRASTRUCTURE ONLY: used to generate the
// golden fixtures in tests/golden/.  Declarations restate the definitions'
// signatures (stochasticSPDP.cpp:940, :549, :1775, :336).
#include <random>
#include <vector>
#include <iostream>
#include <sstream>
#include <cstring>
#include <omp.h>
using std::vector;

void percolationDornic_2D(vector<vector<double>>& Rho, vector<double>& t_meas, double Rh0[], double t_max,
                          double a, double b, double D, double sigma, double dt, double dx, int r, int g);
void percNoDiff_2D(vector<vector<double>>& Rho, vector<double>& t_stop, double Rh0[], double t_max, double a,
                   double b, double D, double dt, double dx, int r, int g);
void RK4_Integrate(vector<double>& Rho_t, double a, double b, double c, double D, double t, double dt, double dx, int g);
vector<double> logarithm10_time_bins(double t_max, double dt);

namespace {
struct Mute {  // the reference prints progress to std::cout; keep it quiet
    std::streambuf* old;
    std::ostringstream sink;
    Mute() : old(std::cout.rdbuf(sink.rdbuf())) {}
    ~Mute() { std::cout.rdbuf(old); }
};
// a stream buffer that drops everything and keeps no state, so threads may share it
struct NullBuf : std::streambuf {
    int overflow(int c) override { return c; }
    std::streamsize xsputn(const char*, std::streamsize n) override { return n; }
};
}

extern "C" {

// One call of percolationDornic_2D; rows are {a, L, t, mean, var, #surv, #active, surv_alt}.
// Returns the number of rows written (<= max_rows) or -1.
int ref_percolation_dornic(const double* t_meas, int n_meas, const double* rho0, double t_max, double a, double b,
                           double D, double sigma, double dt, double dx, int r, int g, double* rows, int max_rows)
{
    Mute m;
    vector<vector<double>> out;
    vector<double> tm(t_meas, t_meas + n_meas);
    vector<double> r0(rho0, rho0 + (size_t)g * g);
    percolationDornic_2D(out, tm, r0.data(), t_max, a, b, D, sigma, dt, dx, r, g);
    int n = 0;
    for (auto& row : out) {
        if (n >= max_rows) break;
        for (int k = 0; k < 8; ++k) rows[n * 8 + k] = k < (int)row.size() ? row[k] : 0.0;
        ++n;
    }
    return n;
}

// The reference's parallel model (critical_exp_delta, stochasticSPDP.cpp:1343-1369):
// one OpenMP thread per value of a, each running percolationDornic_2D (r = 1) from
// the same start.  Returns the wall time in seconds.
double ref_percolation_dornic_par(const double* t_meas, int n_meas, const double* rho0, double t_max, const double* a,
                                  int n_a, double b, double D, double sigma, double dt, double dx, int g, int threads)
{
    NullBuf null;
    std::streambuf* old = std::cout.rdbuf(&null);
    const vector<double> tm(t_meas, t_meas + n_meas);
    const double t0 = omp_get_wtime();
#pragma omp parallel for num_threads(threads) schedule(dynamic, 1)
    for (int i = 0; i < n_a; ++i) {
        vector<vector<double>> out;
        vector<double> tmi = tm;
        vector<double> r0(rho0, rho0 + (size_t)g * g);
        percolationDornic_2D(out, tmi, r0.data(), t_max, a[i], b, D, sigma, dt, dx, 1, g);
    }
    const double sec = omp_get_wtime() - t0;
    std::cout.rdbuf(old);
    return sec;
}

// percNoDiff_2D: noise-off RK4 with the 4th-order cross Laplacian.  Frames at the
// t_stop times are returned as frames[k*g*g + i].  Returns frames written.
int ref_perc_nodiff(const double* t_stop, int n_stop, const double* rho0, double t_max, double a, double b, double D,
                    double dt, double dx, int g, double* frames, int max_frames)
{
    Mute m;
    vector<vector<double>> out;
    vector<double> ts(t_stop, t_stop + n_stop);
    vector<double> r0(rho0, rho0 + (size_t)g * g);
    percNoDiff_2D(out, ts, r0.data(), t_max, a, b, D, dt, dx, 1, g);
    // rows: {a, replicate, t, site, value}
    int nf = (int)(out.size() / ((size_t)g * g));
    if (nf > max_frames) nf = max_frames;
    for (int f = 0; f < nf; ++f)
        for (int i = 0; i < g * g; ++i) frames[(size_t)f * g * g + i] = out[(size_t)f * g * g + i][4];
    return nf;
}

// stochasticSPDP.cpp RK4_Integrate: local RK4 of -b rho^2 - c rho^3 in place.
void ref_rk4_first_order(double* rho, int g, double a, double b, double c, double D, double t, double dt, double dx)
{
    Mute m;
    vector<double> v(rho, rho + (size_t)g * g);
    RK4_Integrate(v, a, b, c, D, t, dt, dx, g);
    std::memcpy(rho, v.data(), sizeof(double) * g * g);
}

// n draws from the libstdc++ distributions the reference's Dornic step constructs
// (stochasticSPDP.cpp:1055-1059): kind 0 std::poisson_distribution<int>(param),
// kind 1 std::gamma_distribution<double>(param, 1), from std::mt19937_64(seed).
int ref_libstdcxx_draws(int kind, double param, unsigned long long seed, int n, double* out)
{
    std::mt19937_64 rng(seed);
    for (int i = 0; i < n; ++i) {
        if (kind == 0) {
            std::poisson_distribution<int> d(param);
            out[i] = (double)d(rng);
        } else {
            std::gamma_distribution<double> d(param, 1.0);
            out[i] = d(rng);
        }
    }
    return n;
}

// The whole draw of the reference's Dornic step (stochasticSPDP.cpp:1053-1059):
// a libstdc++ Poisson count of mean m, then a libstdc++ Gamma of shape mu1 plus
// that count, both from one seeded mt19937_64 (the scale 1/lambda left out).
int ref_libstdcxx_dornic(double m, double mu1, unsigned long long seed, int n, double* out)
{
    std::mt19937_64 rng(seed);
    for (int i = 0; i < n; ++i) {
        std::poisson_distribution<int> pd(m);
        const int count = pd(rng);
        std::gamma_distribution<double> gd(mu1 + count, 1.0);
        out[i] = gd(rng);
    }
    return n;
}

int ref_logarithm10_time_bins(double t_max, double dt, double* out, int max_n)
{
    Mute m;
    vector<double> v = logarithm10_time_bins(t_max, dt);
    int n = (int)v.size() < max_n ? (int)v.size() : max_n;
    for (int i = 0; i < n; ++i) out[i] = v[i];
    return (int)v.size();
}
}
