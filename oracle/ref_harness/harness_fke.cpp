// C-callable harness around the reference's FKE advection-diffusion of the
// consumer species (simulations/Rietkerk_FPE/rietkerk_bjork_FKE.cpp:3614-3695,
// parameters :195-338, stencils :1735-1749 and :3764-3772), built with -DSPB=2
// (vegetation + grazer) and the exprtk stand-in.  TEST INFRASTRUCTURE ONLY.
#include "rietkerk_bjork_basic.h"

extern "C" {
// One advdiff_FKE_MultiSp call on the grazer field (species 1).  Writes the
// moved field to out and the stencils / bounds / prefactor the reference used.
int ref_fke_advdiff(const double* rho, const double* gam, const double* vx, const double* vy, int L, double Dg,
                    double vg, double sigma_g, double dt_adv, double dx, double* out, double* gD, int* RD,
                    double* gV, int* RV, double* pref, int max_stencil)
{
    std::ostringstream sink;
    std::streambuf* old = std::cout.rdbuf(sink.rdbuf());
    double D[Sp] = {0.0, Dg, 0.0, 0.0};
    double v[SpB] = {0.0, vg};
    double dtAdv[SpB] = {0.0, dt_adv};
    set_global_FKE_params(D, v, dtAdv, dt_adv, dx, L, 4);
    const size_t n = (size_t)L * L;
    D2Vec_Double Rho_t(Sp, std::vector<double>(n, 0.0)), Rho_tsar(Sp, std::vector<double>(n, 0.0));
    D2Vec_Double gamma(SpB, std::vector<double>(n, 0.0));
    D2Vec_Pair_Double v_eff(SpB, std::vector<std::pair<double, double>>(n, {0.0, 0.0}));
    for (size_t i = 0; i < n; ++i) {
        Rho_t[1][i] = rho[i];
        gamma[1][i] = gam[i];
        v_eff[1][i] = {vx[i], vy[i]};
    }
    double sig[SpB] = {0.0, sigma_g};
    D2Vec_Double sD(SpB, std::vector<double>(1, 0.0)), sV(SpB, std::vector<double>(1, 0.0));
    sD[1] = precompute_gaussian(sig[1], sig_D_ScaledBounds[1]);
    sV[1] = precompute_gaussian(sig[1], sig_vD_ScaledBounds[1].first);
    advdiff_FKE_MultiSp(Rho_t, Rho_tsar, gamma, v_eff, sD, sV, L);
    std::cout.rdbuf(old);
    for (size_t i = 0; i < n; ++i) out[i] = Rho_t[1][i];
    *RD = sig_D_ScaledBounds[1];
    *RV = sig_vD_ScaledBounds[1].first;
    *pref = mu_vel_prefactor[1];
    if ((int)sD[1].size() > max_stencil || (int)sV[1].size() > max_stencil) return -1;
    for (size_t k = 0; k < sD[1].size(); ++k) gD[k] = sD[1][k];
    for (size_t k = 0; k < sV[1].size(); ++k) gV[k] = sV[1][k];
    return sig_vD_ScaledBounds[1].first == sig_vD_ScaledBounds[1].second ? 0 : 1;
}
}
