// C-callable harness around the reference's Rietkerk step functions
// (simulations/Rietkerk_FPE/rietkerk_bjork_FKE.cpp, built with -DSPB=1 and the
// exprtk stand-in).  TEST INFRASTRUCTURE ONLY.  Declarations restate the
// definitions' signatures (rietkerk_bjork_FKE.cpp:1795, :2393, :1634, :1656, basic.h:302).
#include <vector>
#include <iostream>
#include <sstream>
#include <cstring>
#include <cmath>
#include <cstdint>
#include <random>
using std::vector;
typedef vector<vector<double>> D2;
typedef vector<vector<vector<int>>> D3I;

void RK4_Integrate(D2& Rho_t, D2& Rho_tsar, D3I& nR2, double a, double c, double gmax, double alpha, double d,
                   double rW, double W0, double D[], double K[], double t, double dt, double dx, int g);
void RK4_Integrate_Stochastic_1Sp(D2& Rho_t, D2& Rho_tsar, D2& K1, D2& K2, D2& K3, D2& K4, D3I& nR2, double a,
                                  double c, double gmax, double alpha, double rW, double W0, double (&Dxd2)[3],
                                  double (&K)[3], double t, double dt, double dx, int g);
void determine_neighbours_Sq4(int g, D3I& n);
void determine_neighbours_Sq8(int g, D3I& n);
void set_global_system_params(double dt, double dx);

namespace {
struct Mute {
    std::streambuf* old;
    std::ostringstream sink;
    Mute() : old(std::cout.rdbuf(sink.rdbuf())) {}
    ~Mute() { std::cout.rdbuf(old); }
};
D2 unpack(const double* f, int g) {
    size_t n = (size_t)g * g;
    D2 v(3, vector<double>(n));
    for (int s = 0; s < 3; ++s) std::memcpy(v[s].data(), f + s * n, sizeof(double) * n);
    return v;
}
void pack(const D2& v, double* f, int g) {
    size_t n = (size_t)g * g;
    for (int s = 0; s < 3; ++s) std::memcpy(f + s * n, v[s].data(), sizeof(double) * n);
}
}

extern "C" {

// n_steps of the noise-off model (f_2D + RK4_Integrate, 5-point Laplacian via Sq8)
// applied in place to f = [P|W|O].
void ref_rk_det_steps(double* f, int g, int n_steps, double R, double c, double gmax, double alpha, double d,
                      double rW, double W0, double DP, double DW, double DO, double k1, double k2, double dt, double dx)
{
    Mute m;
    D3I nR2((size_t)g * g, vector<vector<int>>(3, vector<int>(3, 0)));
    determine_neighbours_Sq8(g, nR2);
    double D[3] = {DP, DW, DO};
    double K[3] = {0.0, k1, k2};
    D2 rho = unpack(f, g);
    D2 tsar = rho;
    double t = 0;
    for (int s = 0; s < n_steps; ++s) {
        tsar = rho;
        RK4_Integrate(rho, tsar, nR2, R, c, gmax, alpha, d, rW, W0, D, K, t, dt, dx, g);
        t += dt;
    }
    pack(rho, f, g);
}

// n_steps of the reference's stochastic Rietkerk step on f = [P|W|O], in place, for
// one replicate: the P-Dornic loop of rietkerk_DorFPE_2D_MultiSp
// (rietkerk_bjork_FKE.cpp:4155-4195: skip, Poisson above/below 100, Gamma above/below
// 100, with the constants of :3846-3849) restated here -- the simulation function around it
// cannot run without exprtk -- with the reference's libstdc++ distributions and one
// std::mt19937_64 per replicate; then the reference's own compiled
// RK4_Integrate_Stochastic_1Sp (:2393) for the remainder; then the clamp and the
// DRho update (:4460-4462).  A fixed sample of the reference's ensemble.
void ref_rk_stoch_steps(double* f, int g, int n_steps, unsigned long long seed, double R, double c, double gmax,
                        double alpha, double d, double rW, double W0, double DP, double DW, double DO, double k1,
                        double k2, double sigma, double dt, double dx, double epsilon)
{
    Mute m;
    set_global_system_params(dt, dx);
    D3I nR2((size_t)g * g, vector<vector<int>>(2, vector<int>(2, 0)));
    determine_neighbours_Sq4(g, nR2);
    const size_t n = (size_t)g * g;
    const double dx2 = dx * dx;
    const double beta = -d - 4 * DP / dx2;
    const double lambda_exp = std::exp(beta * dt);
    const double lambda = 2 * beta / (sigma * sigma * (lambda_exp - 1.0));
    const double diff0 = DP / dx2, sigma2_1 = 1 / (sigma * sigma);
    double Dxd2[3] = {diff0, DW / dx2, DO / dx2};
    double K[3] = {0.0, k1, k2};
    std::mt19937_64 rng(seed);
    std::normal_distribution<double> norm(0.0, 1.0);
    D2 rho = unpack(f, g);
    D2 drho = rho;
    D2 tsar(3, vector<double>(n)), K1(3, vector<double>(n)), K2 = K1, K3 = K1, K4 = K1;
    double t = 0.0;
    for (int st = 0; st < n_steps; ++st) {
        for (size_t i = 0; i < n; ++i) {
            const double alpha_i = diff0 * (drho[0][nR2[i][0][0]] + drho[0][nR2[i][0][1]] + drho[0][nR2[i][1][0]] +
                                            drho[0][nR2[i][1][1]]);
            if (alpha_i == 0 && drho[0][i] == 0) continue;
            const double mu = -1.0 + 2.0 * alpha_i * sigma2_1;
            const double ziggy = lambda * lambda_exp * rho[0][i];
            double gru;
            if (ziggy == 0.0) {
                gru = mu + 1.0;
            } else if (ziggy > 100) {
                const long gauss = long(norm(rng) * std::sqrt(ziggy) + ziggy);
                gru = mu + 1.0 + gauss;
            } else {
                std::poisson_distribution<int> poisson(ziggy);
                gru = mu + 1.0 + poisson(rng);
            }
            if (gru > 100) {
                rho[0][i] = (norm(rng) * std::sqrt(gru) + gru) / lambda;
            } else {
                std::gamma_distribution<double> gamma_distr(gru, 1.0);
                rho[0][i] = gamma_distr(rng) / lambda;
            }
        }
        RK4_Integrate_Stochastic_1Sp(rho, tsar, K1, K2, K3, K4, nR2, R, c, gmax, alpha, rW, W0, Dxd2, K, t, dt, dx, g);
        for (int s = 0; s < 3; ++s)
            for (size_t i = 0; i < n; ++i) {
                if (rho[s][i] < epsilon && rho[s][i] >= 0.0) rho[s][i] = 0.0;
                drho[s][i] = rho[s][i];
            }
        t += dt;
    }
    pack(rho, f, g);
}

// One call of the stochastic remainder RK4 (f_2Dor, Sq4) on f = [P*|W|O], in place.
void ref_rk_stoch_remainder(double* f, int g, double R, double c, double gmax, double alpha, double rW, double W0,
                            double DW, double DO, double k1, double k2, double dt, double dx)
{
    Mute m;
    set_global_system_params(dt, dx);
    D3I nR2((size_t)g * g, vector<vector<int>>(2, vector<int>(2, 0)));
    determine_neighbours_Sq4(g, nR2);
    size_t n = (size_t)g * g;
    double Dxd2[3] = {0.0, DW / (dx * dx), DO / (dx * dx)};
    double K[3] = {0.0, k1, k2};
    D2 rho = unpack(f, g);
    D2 tsar(3, vector<double>(n)), K1(3, vector<double>(n)), K2 = K1, K3 = K1, K4 = K1;
    RK4_Integrate_Stochastic_1Sp(rho, tsar, K1, K2, K3, K4, nR2, R, c, gmax, alpha, rW, W0, Dxd2, K, 0.0, dt, dx, g);
    pack(rho, f, g);
}
}
