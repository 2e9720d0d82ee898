// C-callable harness around the reference's Rietkerk step functions
// (simulations/Rietkerk_FPE/rietkerk_bjork_FKE.cpp, built with -DSPB=1 and the
// exprtk stand-in).  TEST INFRASTRUCTURE ONLY.  Declarations restate the
// definitions' signatures (rietkerk_bjork_FKE.cpp:1795, :2393, :1634, :1656, basic.h:302).
#include <vector>
#include <iostream>
#include <sstream>
#include <cstring>
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
