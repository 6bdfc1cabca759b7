// Test-oracle harness around the CIFlow reference sources (compiled unmodified
// from the reference tree by oracle/Makefile into oracle/_ref/).
//
// This file is test infrastructure: only tests/, the smoke check and the CPU
// baseline of bench.py load the library it builds. It exposes the reference's
// own classes through a plain C API so that Python can:
//   * build a Hamiltonian in memory (Hamiltonian(L,0,nup,ndown,Econst) plus
//     setTmat/setVmat, Hamiltonian.cpp:77-113,255-320) or read a psi4 text dump
//     (Hamiltonian(filename), Hamiltonian.cpp:157-171,707-885);
//   * construct FCI/DOCI, which builds the upper-triangle CRS in the constructor
//     (CIMethod.cpp:566-580 -> build_parallel :489-561);
//   * read back the CRS arrays data/col/row (SparseMatrix_CRS.h:107-111);
//   * call the reference SparseMatrix_CRS_Sym::mvprod (SparseMatrix_CRS.cpp:700-723)
//     so scipy's ARPACK can drive the reference matvec;
//   * install an eigenvector and run CIDens::construct_density
//     (CIMethod.cpp:161-171, CIDens.cpp:323-334) and read the RDMs through
//     get_one_rdm/get_two_rdm (CIDens.cpp:166-292);
//   * build FCI_File from a determinant file and read back its list;
//   * apply Jacobi rotations with OrbitalTransform::do_jacobi_rotation
//     (OrbitalTransform.cpp:278-414) and read the rotated integrals and the
//     accumulated unitary (UnitaryMatrix::get_full_transformation, UnitaryMatrix.cpp:167-183);
//   * evaluate DensDOCI::find_min_angle / calc_rotate (CIDens.cpp:1279-1464) for
//     every orbital pair, with the pair selection of LocalMinimizer::scan_orbitals
//     (LocalMinimizer.cpp:89-118).
#include <cmath>
#include <cstring>
#include <fstream>
#include <functional>
#include <iomanip>
#include <iostream>
#include <memory>
#include <string>
#include <vector>

// Members the harness reads (CIMethod::_mat, SparseMatrix_CRS::data/col/row,
// CIMethod::_cid, CIMethod::_solved) are protected in the reference; this TU
// only reads them, with the same class layout.
#define protected public
#include "CIDens.h"
#include "CIMethod.h"
#include "Hamiltonian.h"
#include "Output.h"
#include "SparseMatrix_CRS.h"
#undef protected
#include "OrbitalTransform.h"
#include "Permutator.h"
#include "UnitaryMatrix.h"

namespace {

struct RefCI {
    Hamiltonian *ham = nullptr;
    CIMethod *cim = nullptr;
    int method = 0;  // 0 = FCI, 1 = DOCI
};

Hamiltonian *make_ham(int L, int nup, int ndown, double econst, const double *h, const double *eri) {
    Hamiltonian *ham = new Hamiltonian(L, 0, nup, ndown, econst);
    for (int i = 0; i < L; ++i)
        for (int j = 0; j < L; ++j) ham->setTmat(i, j, h[i * L + j]);
    // eri is chemist (ij|kl), row-major L^4; the reference stores physics
    // <ik|jl> = (ij|kl) exactly as its text reader does (Hamiltonian.cpp:873).
    const size_t L1 = L, L2 = L1 * L1, L3 = L2 * L1;
    for (int i = 0; i < L; ++i)
        for (int j = 0; j < L; ++j)
            for (int k = 0; k < L; ++k)
                for (int l = 0; l < L; ++l) ham->setVmat(i, k, j, l, eri[i * L3 + j * L2 + k * L1 + l]);
    return ham;
}

}  // namespace

extern "C" {

// Reads a psi4 integral dump with the reference reader. Call once with h == NULL
// to obtain L/nup/ndown/econst, then again with h (L*L) and eri (L^4, chemist).
int ref_ham_read_file(const char *filename, int *L, int *nup, int *ndown, double *econst, double *h,
                      double *eri) {
    Hamiltonian ham{std::string(filename)};
    *L = ham.getL();
    *nup = ham.getnup();
    *ndown = ham.getndown();
    *econst = ham.getEconst();
    if (!h) return 0;
    const int n = *L;
    const size_t L1 = n, L2 = L1 * L1, L3 = L2 * L1;
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) h[i * n + j] = ham.getTmat(i, j);
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j)
            for (int k = 0; k < n; ++k)
                for (int l = 0; l < n; ++l) eri[i * L3 + j * L2 + k * L1 + l] = ham.getVmat(i, k, j, l);
    return 0;
}

// method 0 = FCI, 1 = DOCI. When filename is non-NULL the Hamiltonian comes from
// the reference text reader (with its point-group irreps); otherwise from h/eri.
void *ref_ci_create(int method, const char *filename, int L, int nup, int ndown, double econst,
                    const double *h, const double *eri) {
    RefCI *r = new RefCI;
    r->method = method;
    r->ham = filename ? new Hamiltonian(std::string(filename)) : make_ham(L, nup, ndown, econst, h, eri);
    if (method == 0)
        r->cim = new FCI(r->ham);
    else
        r->cim = new DOCI(r->ham);
    return r;
}

void ref_ci_destroy(void *p) {
    RefCI *r = static_cast<RefCI *>(p);
    delete r->cim;
    delete r->ham;
    delete r;
}

long long ref_ci_dim(void *p) { return static_cast<RefCI *>(p)->cim->get_dim(); }
long long ref_ci_nnz(void *p) { return static_cast<RefCI *>(p)->cim->_mat.data.size(); }

// Copies the reference CRS: row (dim+1), col (nnz), val (nnz).
void ref_ci_export(void *p, unsigned *row, unsigned *col, double *val) {
    const SparseMatrix_CRS &m = static_cast<RefCI *>(p)->cim->_mat;
    std::memcpy(row, m.row.data(), m.row.size() * sizeof(unsigned));
    std::memcpy(col, m.col.data(), m.col.size() * sizeof(unsigned));
    std::memcpy(val, m.data.data(), m.data.size() * sizeof(double));
}

// The reference matvec y = (U + U^T - D) x, serial (SparseMatrix_CRS.cpp:700-723).
void ref_ci_mvprod(void *p, const double *x, double *y) {
    static_cast<RefCI *>(p)->cim->_mat.mvprod(x, y);
}

// Installs eigenpair (e without Econst, c of length dim) and builds the RDMs
// with the reference CIDens (DensFCI / DensDOCI). rdm1: [2][L][L];
// rdm2_aa/bb: [npair][npair] with pair(p<q) = p*L+q-(p+1)(p+2)/2; rdm2_ab: [L*L][L*L].
// Returns CIDens::get_dens_energy().
double ref_ci_density(void *p, double e, const double *c, double *rdm1, double *rdm2_aa, double *rdm2_ab,
                      double *rdm2_bb) {
    RefCI *r = static_cast<RefCI *>(p);
    CIMethod *cim = r->cim;
    const int dim = cim->get_dim();
    cim->_eigval = matrix(1, 1);
    cim->_eigval(0, 0) = e;
    cim->_eigvec = matrix(dim, 1);
    for (int i = 0; i < dim; ++i) cim->_eigvec(i, 0) = c[i];
    cim->_solved = true;
    cim->_cid->reset_density();
    cim->construct_density(0, true);
    CIDens *d = cim->_cid.get();
    const int L = cim->get_l();
    for (int s = 0; s < 2; ++s)
        for (int i = 0; i < L; ++i)
            for (int j = 0; j < L; ++j) rdm1[(s * L + i) * L + j] = d->get_one_rdm(s, i, j);
    const int np = L * (L - 1) / 2;
    for (int p_ = 0; p_ < L; ++p_)
        for (int q = p_ + 1; q < L; ++q)
            for (int r_ = 0; r_ < L; ++r_)
                for (int s = r_ + 1; s < L; ++s) {
                    const int a = p_ * L + q - (p_ + 1) * (p_ + 2) / 2;
                    const int b = r_ * L + s - (r_ + 1) * (r_ + 2) / 2;
                    rdm2_aa[a * np + b] = d->get_two_rdm(0, p_, q, r_, s);
                    rdm2_bb[a * np + b] = d->get_two_rdm(2, p_, q, r_, s);
                }
    const int L2 = L * L;
    for (int p_ = 0; p_ < L; ++p_)
        for (int q = 0; q < L; ++q)
            for (int r_ = 0; r_ < L; ++r_)
                for (int s = 0; s < L; ++s)
                    rdm2_ab[(p_ * L + q) * L2 + r_ * L + s] = d->get_two_rdm(1, p_, q, r_, s);
    return d->get_dens_energy();
}

// Installs eigenpair (e without Econst, c) as ref_ci_density does.
static void install(CIMethod *cim, double e, const double *c) {
    const int dim = cim->get_dim();
    cim->_eigval = matrix(1, 1);
    cim->_eigval(0, 0) = e;
    cim->_eigvec = matrix(dim, 1);
    for (int i = 0; i < dim; ++i) cim->_eigvec(i, 0) = c[i];
    cim->_solved = true;
}

// The CI-vector block of the reference output (OutputSFFCI / OutputSFDOCI /
// OutputSFFCI_File::print_ci_vec, Output.cpp:190-263) for eigenpair (e, c), written
// to `path` with the precision the reference's report has there (16).
int ref_print_civec(void *p, double e, const double *c, double nauw, const char *path) {
    CIMethod *cim = static_cast<RefCI *>(p)->cim;
    install(cim, e, c);
    OutputSingleFile *o = cim->_output.get();
    o->_file.open(path, std::ios::out);
    if (!o->_file.is_open()) return -1;
    o->_file.precision(16);
    o->print_ci_vec(0, nauw);
    o->_file.close();
    return 0;
}

// The RDM text of CIMethod::print_one_rdm / print_two_rdm (CIMethod.cpp:184-195,
// CIDens.cpp:978-1026) for eigenpair (e, c), precision 16 as OutputSingleFile::print_rdm.
int ref_print_rdm(void *p, double e, const double *c, const char *path) {
    CIMethod *cim = static_cast<RefCI *>(p)->cim;
    install(cim, e, c);
    cim->_cid->reset_density();
    cim->construct_density(0, true);
    std::ofstream f(path);
    if (!f.is_open()) return -1;
    f.precision(16);
    cim->print_one_rdm(f);
    cim->print_two_rdm(f);
    return 0;
}

// FCI_File(ham, det_file) (CIMethod.cpp:890-919): the Hamiltonian from a psi4 text
// dump (ham_file) or from h/eri, the determinant list read by Permutator_File
// (Permutator.cpp:179-224); the CRS is built by the constructor. Works with the
// ref_ci_* accessors above.
void *ref_file_ci_create(const char *ham_file, int L, int nup, int ndown, double econst, const double *h,
                         const double *eri, const char *det_file) {
    RefCI *r = new RefCI;
    r->method = 2;
    r->ham = ham_file ? new Hamiltonian(std::string(ham_file)) : make_ham(L, nup, ndown, econst, h, eri);
    r->cim = new FCI_File(r->ham, std::string(det_file));
    return r;
}

// The determinant list of a FCI_File object in list order (64-bit strings).
void ref_file_dets(void *p, unsigned long long *up, unsigned long long *down) {
    CIMethod *cim = static_cast<RefCI *>(p)->cim;
    Permutator *perm = cim->get_perm();
    const int n = perm->get_dim();
    TYPE det[2];
    for (int i = 0; i < n; ++i) {
        perm->permutate_bit(det, i);
        up[i] = (unsigned long long)det[0];
        down[i] = (unsigned long long)det[1];
    }
}

// Applies nrot Jacobi rotations in order to the Hamiltonian built from h/eri
// (OrbitalTransform::do_jacobi_rotation on the same Hamiltonian object, as the
// optimisers do). Outputs: h_out (L*L), eri_out (L^4 chemist), U_out (L*L
// row-major: U[a*L+p] = row a of the reference unitary).
int ref_jacobi(int L, int nup, int ndown, double econst, const double *h, const double *eri, int nrot, const int *k,
               const int *l, const double *theta, double *h_out, double *eri_out, double *U_out) {
    Hamiltonian *ham = make_ham(L, nup, ndown, econst, h, eri);
    {
        OrbitalTransform tr(ham);
        for (int i = 0; i < nrot; ++i) tr.do_jacobi_rotation(k[i], l[i], theta[i], ham);
        const std::vector<double> u = tr.get_unitary().get_full_transformation();  // column-major
        for (int a = 0; a < L; ++a)
            for (int p_ = 0; p_ < L; ++p_) U_out[a * L + p_] = u[a + (size_t)L * p_];
    }
    const size_t L1 = L, L2 = L1 * L1, L3 = L2 * L1;
    for (int i = 0; i < L; ++i)
        for (int j = 0; j < L; ++j) h_out[i * L + j] = ham->getTmat(i, j);
    for (int i = 0; i < L; ++i)
        for (int j = 0; j < L; ++j)
            for (int k_ = 0; k_ < L; ++k_)
                for (int l_ = 0; l_ < L; ++l_) eri_out[i * L3 + j * L2 + k_ * L1 + l_] = ham->getVmat(i, k_, j, l_);
    delete ham;
    return 0;
}

// OrbitalTransform::fillHamCI (OrbitalTransform.cpp:64-135) with the unitary set to
// U (row-major, U[a*L + p]: row a is the new orbital a in the old orbitals; the
// reference block is column-major, element (a, p) at a + L*p). Outputs the
// rotated h (L*L) and eri (L^4, chemist) the reference Hamiltonian holds.
int ref_rotate(int L, int nup, int ndown, double econst, const double *h, const double *eri, const double *U,
               double *h_out, double *eri_out) {
    Hamiltonian *ham = make_ham(L, nup, ndown, econst, h, eri);
    Hamiltonian *rot = make_ham(L, nup, ndown, econst, h, eri);
    {
        OrbitalTransform tr(ham);
        double *blk = tr.get_unitary().getBlock(0);
        for (int a = 0; a < L; ++a)
            for (int p_ = 0; p_ < L; ++p_) blk[a + (size_t)L * p_] = U[a * L + p_];
        tr.fillHamCI(*rot);
    }
    const size_t L1 = L, L2 = L1 * L1, L3 = L2 * L1;
    for (int i = 0; i < L; ++i)
        for (int j = 0; j < L; ++j) h_out[i * L + j] = rot->getTmat(i, j);
    for (int i = 0; i < L; ++i)
        for (int j = 0; j < L; ++j)
            for (int k_ = 0; k_ < L; ++k_)
                for (int l_ = 0; l_ < L; ++l_) eri_out[i * L3 + j * L2 + k_ * L1 + l_] = rot->getVmat(i, k_, j, l_);
    delete rot;
    delete ham;
    return 0;
}

// DOCI pair scan with the reference density of the installed eigenpair (as in
// ref_ci_density). For pair index P of k < l: theta/energy/found as
// LocalMinimizer::scan_orbitals decides them (start 0.3, then 0.01 on a maximum;
// found = minimum with |theta| <= pi/2), energy = calc_rotate(theta). fixed_energy
// [P * nfixed + i] = calc_rotate(k, l, fixed[i]) pins the energy expression alone.
int ref_doci_scan(void *p, double e, const double *c, double *theta, double *energy, int *found, int nfixed,
                  const double *fixed, double *fixed_energy) {
    RefCI *r = static_cast<RefCI *>(p);
    if (r->method != 1) return -1;
    CIMethod *cim = r->cim;
    const int dim = cim->get_dim();
    cim->_eigval = matrix(1, 1);
    cim->_eigval(0, 0) = e;
    cim->_eigvec = matrix(dim, 1);
    for (int i = 0; i < dim; ++i) cim->_eigvec(i, 0) = c[i];
    cim->_solved = true;
    cim->_cid->reset_density();
    cim->construct_density(0, true);
    const DensDOCI *d = dynamic_cast<const DensDOCI *>(cim->_cid.get());
    if (!d) return -2;
    Hamiltonian &ham = *r->ham;
    std::function<double(int, int)> T = [&ham](int a, int b) -> double { return ham.getTmat(a, b); };
    std::function<double(int, int, int, int)> V = [&ham](int a, int b, int c_, int d_) -> double {
        return ham.getVmat(a, b, c_, d_);
    };
    const int L = cim->get_l();
    int P = 0;
    for (int k = 0; k < L; ++k)
        for (int l = k + 1; l < L; ++l, ++P) {
            std::pair<double, bool> f = d->find_min_angle(k, l, 0.3, T, V);
            if (!f.second) f = d->find_min_angle(k, l, 0.01, T, V);
            theta[P] = f.first;
            energy[P] = d->calc_rotate(k, l, f.first, T, V);
            found[P] = (f.second && std::fabs(f.first) <= M_PI / 2.0) ? 1 : 0;
            for (int i = 0; i < nfixed; ++i) fixed_energy[P * nfixed + i] = d->calc_rotate(k, l, fixed[i], T, V);
        }
    return 0;
}

}  // extern "C"
