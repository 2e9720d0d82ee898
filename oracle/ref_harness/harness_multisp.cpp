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
void save_frame(D2& Rho_t, const std::string& parendir, const std::string& filenamePattern, double a, double a_st,
                double a_end, double t, double dt, double dx, double dP, int r, int g, std::string header,
                bool overwrite);
void save_prelimframe(D2& Rho_t, const std::string& parendir, const std::string& filenamePattern, double a,
                      double a_st, double a_end, double t, double dt, double dx, double dP, int r, int g,
                      std::string header, bool overwrite, bool delete_previous);

extern "C" {
// save_frame (multiSPDP.cpp:1596-1643) of one field of g*g values.
void ref_save_frame(const double* rho, int g, const char* parendir, const char* pattern, double a, int r,
                    const char* header)
{
    std::ostringstream sink;
    std::streambuf* old = std::cout.rdbuf(sink.rdbuf());
    D2 R(1, std::vector<double>(rho, rho + (size_t)g * g));
    save_frame(R, parendir, pattern, a, 0.0, 0.0, 0.0, 0.1, 1.0, 0.0, r, g, header, false);
    std::cout.rdbuf(old);
}
// save_prelimframe (multiSPDP.cpp:1493-1594) of n rows {t, mean, var, surv, active}.
void ref_save_prelim(const double* rows, int n, int g, const char* parendir, const char* pattern, double a, int r,
                     const char* header)
{
    std::ostringstream sink;
    std::streambuf* old = std::cout.rdbuf(sink.rdbuf());
    D2 R(n, std::vector<double>(5));
    for (int i = 0; i < n; ++i)
        for (int k = 0; k < 5; ++k) R[i][k] = rows[i * 5 + k];
    save_prelimframe(R, parendir, pattern, a, 0.0, 0.0, 0.0, 0.1, 1.0, 0.0, r, g, header, false, false);
    std::cout.rdbuf(old);
}

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
