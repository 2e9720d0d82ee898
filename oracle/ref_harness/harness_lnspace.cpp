// TEST INFRASTRUCTURE ONLY (golden fixtures).  The reference's lnspace<int>
// (simulations/Percolation_FD/stochasticSPDP.cpp:281-301) is a template that the
// reference's own object file inlines into its one caller, so no symbol of it
// exists to call.  This translation unit compiles the reference source where it
// lies and instantiates the template it defines, unchanged.
#include "stochasticSPDP.cpp"

template std::vector<double> lnspace<int>(int, int, int);

extern "C" int ref_lnspace(int start, int end, int num, double* out, int max_n)
{
    std::vector<double> v = lnspace<int>(start, end, num);
    int n = (int)v.size() < max_n ? (int)v.size() : max_n;
    for (int i = 0; i < n; ++i) out[i] = v[i];
    return (int)v.size();
}
