// C-callable harness around the reference's MultiSp DP remainder
// (simulations/Percolation_FD/multiSPDP.cpp, built with -DSPB=1 and the exprtk
// stand-in).  TEST INFRASTRUCTURE ONLY.  Declarations restate the definitions'
// signatures (multiSPDP.cpp:1821, :164).
#include <vector>
#include <iostream>
#include <sstream>
#include <cstring>
using std::vector;
typedef vector<vector<double>> D2;
typedef vector<vector<vector<int>>> D3I;

void RK4_Integrate_Stochastic_MultiSp(D2& Rho_t, D2& Rho_tsar, D2& K1, D2& K2, D2& K3, D2& K4, D3I& nR2, double b,
                                      double c, double (&Dxd2)[1], double (&A)[1][1], double (&H)[1][1],
                                      double (&E)[1], double t, double dt, double dx, int g);
void set_global_system_params(double dt, double dx);

extern "C" {
// One call of RK4_Integrate_Stochastic_MultiSp with SPB=1 (f_DP_Dor_1Sp: -b rho^2), in place.
void ref_ms_rk4_remainder(double* rho, int g, double b, double dt, double dx)
{
    std::ostringstream sink;
    std::streambuf* old = std::cout.rdbuf(sink.rdbuf());
    set_global_system_params(dt, dx);
    size_t n = (size_t)g * g;
    D2 R(1, vector<double>(rho, rho + n));
    D2 tsar(1, vector<double>(n)), K1 = tsar, K2 = tsar, K3 = tsar, K4 = tsar;
    D3I nR2(n, vector<vector<int>>(2, vector<int>(2, 0)));
    double Dxd2[1] = {0.0}, A[1][1] = {{0.0}}, H[1][1] = {{0.0}}, E[1] = {0.0};
    RK4_Integrate_Stochastic_MultiSp(R, tsar, K1, K2, K3, K4, nR2, b, 0.0, Dxd2, A, H, E, 0.0, dt, dx, g);
    std::memcpy(rho, R[0].data(), sizeof(double) * n);
    std::cout.rdbuf(old);
}
}
