// A CIFlow-style driver compiled against the C++ façade (include/ciflow_gb300/ciflow.hpp),
// written like the reference's own tests: TestDOCI.cpp (DOCI energy of BeH2) and
// TestDensity.cpp (FCI density energy equals the CI energy). The integrals come
// from a binary file written by tests/test_gpu_facade.py:
//   int32 L, nup, ndown; float64 econst; float64 h[L*L]; float64 eri[L^4] (chemist).
// Prints one JSON line with the results.
#include <ciflow_gb300/ciflow.hpp>

#include <cstdio>
#include <fstream>
#include <vector>

using namespace ciflow_gb300;

int main(int argc, char **argv) {
    if (argc < 2) return 2;
    std::ifstream f(argv[1], std::ios::binary);
    int32_t L = 0, nup = 0, ndown = 0;
    double econst = 0;
    f.read((char *)&L, 4).read((char *)&nup, 4).read((char *)&ndown, 4).read((char *)&econst, 8);
    std::vector<double> h((size_t)L * L), eri((size_t)L * L * L * L);
    f.read((char *)h.data(), h.size() * 8).read((char *)eri.data(), eri.size() * 8);
    if (!f) return 3;

    // Hamiltonian(L, nGroup, nup, ndown, Econst) + setTmat/setVmat, physics <ij|kl> = (ik|jl)
    Hamiltonian ham(L, 0, nup, ndown, econst);
    for (int i = 0; i < L; ++i)
        for (int j = 0; j < L; ++j) ham.setTmat(i, j, h[(size_t)i * L + j]);
    for (int i = 0; i < L; ++i)
        for (int j = 0; j < L; ++j)
            for (int k = 0; k < L; ++k)
                for (int l = 0; l < L; ++l) ham.setVmat(i, k, j, l, eri[(((size_t)i * L + j) * L + k) * L + l]);

    DOCI doci(&ham);
    doci.set_tolerance(1e-10);
    doci.solve();
    const double e_doci = doci.get_ci_energy();

    FCI fci(&ham);
    fci.set_tolerance(1e-10);
    fci.solve();
    fci.construct_density(0, true);
    CIDens *d = fci.density();
    d->test_invariants(true);
    const double e_fci = fci.get_ci_energy(), e_dens = d->get_dens_energy();

    // the CRS view and matvec of the façade
    SparseMatrix_CRS_Sym &m = fci.get_mat();
    std::vector<double> x(m.getn(), 1.0), y(m.getn());
    m.mvprod(x.data(), y.data());
    double ysum = 0;
    for (double v : y) ysum += v;

    FCI mixed(&ham, CIGPU_MIXED);
    mixed.set_tolerance(1e-8);
    mixed.solve();

    std::printf("{\"e_doci\": %.17g, \"e_fci\": %.17g, \"e_dens\": %.17g, \"e_fci_mixed\": %.17g, "
                "\"dim_fci\": %d, \"nnz_upper\": %d, \"h00\": %.17g, \"ysum\": %.17g}\n",
                e_doci, e_fci, e_dens, mixed.get_ci_energy(), fci.get_dim(), m.datasize(), m(0, 0), ysum);
    return 0;
}
