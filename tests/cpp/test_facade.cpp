// A CIFlow-style driver compiled against the C++ façade (include/ciflow_gb300/ciflow.hpp),
// written like the reference's own tests: TestDOCI.cpp (DOCI energy of BeH2) and
// TestDensity.cpp (FCI density energy equals the CI energy). The integrals come
// from a binary file written by tests/test_gpu_facade.py:
//   int32 L, nup, ndown; float64 econst; float64 h[L*L]; float64 eri[L^4] (chemist).
// Prints one JSON line with the results.
#include <ciflow_gb300/ciflow.hpp>

#include <cstdio>
#include <fstream>
#include <string>
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

    // psi4 text dump written and read back (Hamiltonian::save_file / Hamiltonian(filename))
    const std::string dir = argc > 2 ? argv[2] : ".";
    ham.save_file(dir + "/beh2.dat");
    Hamiltonian back(dir + "/beh2.dat");
    int same = back.getL() == L && back.getnup() == nup && back.getEconst() == econst;
    for (int i = 0; i < L && same; ++i)
        for (int j = 0; j < L; ++j) same = same && back.getTmat(i, j) == ham.getTmat(i, j);
    for (size_t k = 0; k < ham.eri().size() && same; ++k) same = same && back.eri()[k] == ham.eri()[k];

    // FCI_File over the full FCI list (alpha-major, colex strings) and CI_Big over the same file
    {
        std::ofstream dets(dir + "/dets.txt");
        dets << "#all determinants\n";
        std::vector<uint64_t> sa, sb;
        for (uint64_t s = 0; s < (1ull << L); ++s) {
            if (__builtin_popcountll(s) == nup) sa.push_back(s);
            if (__builtin_popcountll(s) == ndown) sb.push_back(s);
        }
        auto bits = [&](uint64_t s) {
            std::string out(L, '0');
            for (int o = 0; o < L; ++o)
                if ((s >> o) & 1) out[L - 1 - o] = '1';
            return out;
        };
        for (uint64_t a : sa)
            for (uint64_t b : sb) dets << bits(a) << "|" << bits(b) << "\n";
    }
    FCI_File file_ci(&ham, dir + "/dets.txt");
    file_ci.set_tolerance(1e-10);
    file_ci.solve();
    file_ci.construct_density(0, true);
    const double e_file_dens = file_ci.density()->get_dens_energy();
    CI_Big big(&ham, dir + "/dets.txt");
    big.set_tolerance(1e-10);
    big.solve();
    fci.print_ci_vec(dir + "/fci_vec.txt", 1e-4);
    fci.print_rdm(dir + "/fci_rdm.txt");

    // orbital optimisers on DOCI: a short anneal and the local minimiser
    DOCI opt_ci(&ham);
    opt_ci.set_tolerance(1e-10);
    opt_ci.solve();
    const double e_start = opt_ci.get_ci_energy();
    SimulatedAnnealing sa(&opt_ci, 0.4, 0.99, 1.4, 0.999, 7);
    sa.set_steps(60);
    sa.set_speculate(4);
    sa.optimize();
    sa.set_cim_optimal();
    const double e_sa = opt_ci.get_ci_energy(), e_sa_opt = sa.get_opt_ci_energy();
    LocalMinimizer lm(&opt_ci, 3);
    lm.set_conv_steps(3);
    const double e_lm = lm.optimize();

    std::printf("{\"e_doci\": %.17g, \"e_fci\": %.17g, \"e_dens\": %.17g, \"e_fci_mixed\": %.17g, "
                "\"dim_fci\": %d, \"nnz_upper\": %d, \"h00\": %.17g, \"ysum\": %.17g, \"psi4_round_trip\": %d, "
                "\"e_file\": %.17g, \"e_file_dens\": %.17g, \"e_big\": %.17g, \"dim_file\": %d, "
                "\"e_opt_start\": %.17g, \"e_sa\": %.17g, \"e_sa_opt\": %.17g, \"e_lm\": %.17g, \"e_lm_cim\": %.17g}\n",
                e_doci, e_fci, e_dens, mixed.get_ci_energy(), fci.get_dim(), m.datasize(), m(0, 0), ysum, same,
                file_ci.get_ci_energy(), e_file_dens, big.get_ci_energy(), file_ci.get_dim(), e_start, e_sa, e_sa_opt,
                e_lm, opt_ci.get_ci_energy());
    return 0;
}
