// C++ façade with CIFlow's class names over the cigpu C ABI (header-only).
//
// Code written against CIFlow's lowest-eigenpair API compiles against these
// classes with the same calls:
//   Hamiltonian(L, nGroup=0, nup, ndown, Econst), setTmat/setVmat/getTmat/getVmat
//       (Hamiltonian.h:80-170; physics <ij|kl>, stored as chemist (ik|jl))
//   FCI(ham) / DOCI(ham): the constructor builds the CRS (CIMethod.cpp:566-580)
//   solve(neig=1), get_ci_energy(), get_eigvec(...), set_ham(ham, build),
//       construct_density(state, trdm)                    (CIMethod.h:37-132)
//   SparseMatrix_CRS_Sym: getn/getm/datasize/operator()/mvprod (SparseMatrix_CRS.h:33-130)
//   CIDens / DensFCI / DensDOCI: construct_density, get_one_rdm, get_two_rdm,
//       get_one/two_electron_energy, get_dens_energy, test_invariants (CIDens.h:29-174)
//   Hamiltonian(filename) / save_file (psi4 integral text), FCI_File / CI_Big (determinant
//       lists, CIMethod.h:164-189), print_ci_vec / print_rdm (the reference's text dumps)
//   SimulatedAnnealing / LocalMinimizer (orbital optimisers over cigpu_orbopt)
// Differences by design: errors throw ciflow_gb300::Error (with the cigpu status)
// instead of calling exit(1); solve keeps the CRS resident; FCI/DOCI take an
// optional precision (CIGPU_FP64 = the plain method, CIGPU_MIXED).
#pragma once

#include <cigpu.h>

#include <cmath>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace ciflow_gb300 {

class Error : public std::runtime_error {
   public:
    Error(int status, const std::string &what)
        : std::runtime_error(what + ": " + cigpu_strerror(status)), status_(status) {}
    int status() const { return status_; }

   private:
    int status_;
};

inline void check(int status, const char *what) {
    if (status != CIGPU_OK) throw Error(status, what);
}

inline int64_t binomial(int n, int k) {
    if (k < 0 || k > n) return 0;
    if (k > n - k) k = n - k;
    int64_t r = 1;
    for (int i = 1; i <= k; ++i) r = r * (n - k + i) / i;
    return r;
}

class Hamiltonian {
   public:
    // Hamiltonian(Norbitals, nGroup, nup, ndown, Econstant) (Hamiltonian.cpp:77-113); only C1 (nGroup 0).
    Hamiltonian(int Norbitals, int nGroup, int nup, int ndown, double Econstant)
        : L_(Norbitals), nup_(nup), ndown_(ndown), econst_(Econstant),
          h_((size_t)Norbitals * Norbitals, 0.0), eri_((size_t)Norbitals * Norbitals * Norbitals * Norbitals, 0.0) {
        if (nGroup != 0) throw Error(CIGPU_ENOTSUP, "Hamiltonian: only point group 0 (C1)");
    }
    // Hamiltonian(filename) for a psi4 integral text dump (Hamiltonian.cpp:157-171, 707-885).
    explicit Hamiltonian(const std::string &filename) : L_(0), nup_(0), ndown_(0), econst_(0) {
        check(cigpu_ham_read_psi4(filename.c_str(), &L_, &nup_, &ndown_, &econst_, nullptr, nullptr, nullptr, nullptr),
              "cigpu_ham_read_psi4");
        h_.assign((size_t)L_ * L_, 0.0);
        eri_.assign((size_t)L_ * L_ * L_ * L_, 0.0);
        check(cigpu_ham_read_psi4(filename.c_str(), &L_, &nup_, &ndown_, &econst_, h_.data(), eri_.data(), nullptr,
                                  &hf_energy_),
              "cigpu_ham_read_psi4");
    }
    // Takes ownership of a device Hamiltonian (e.g. an optimiser's rotated one) and reads its integrals.
    explicit Hamiltonian(cigpu_ham *owned, int L, int nup, int ndown, double econst)
        : L_(L), nup_(nup), ndown_(ndown), econst_(econst), h_((size_t)L * L), eri_((size_t)L * L * L * L) {
        dev_.reset(owned);
        check(cigpu_ham_export(owned, h_.data(), eri_.data()), "cigpu_ham_export");
        dirty_ = false;
    }
    // Hamiltonian::save_file's format (C1, 17 significant digits).
    void save_file(const std::string &filename) const {
        check(cigpu_ham_write_psi4(filename.c_str(), L_, nup_, ndown_, econst_, h_.data(), eri_.data(), hf_energy_),
              "cigpu_ham_write_psi4");
    }
    double get_hf_energy() const { return hf_energy_; }
    int getL() const { return L_; }
    int getnup() const { return nup_; }
    int getndown() const { return ndown_; }
    double getEconst() const { return econst_; }
    void setEconst(double v) { econst_ = v; dirty_ = true; }
    double getTmat(int i, int j) const { return h_[(size_t)i * L_ + j]; }
    void setTmat(int i, int j, double v) {
        h_[(size_t)i * L_ + j] = v;
        h_[(size_t)j * L_ + i] = v;
        dirty_ = true;
    }
    // physics <ij|kl> = chemist (ik|jl); sets the 8 symmetry partners
    double getVmat(int i, int j, int k, int l) const { return eri_[idx(i, k, j, l)]; }
    void setVmat(int i, int j, int k, int l, double v) {
        const int p = i, q = k, r = j, s = l;
        const int perm[8][4] = {{p, q, r, s}, {q, p, r, s}, {p, q, s, r}, {q, p, s, r},
                                {r, s, p, q}, {s, r, p, q}, {r, s, q, p}, {s, r, q, p}};
        for (auto &x : perm) eri_[idx(x[0], x[1], x[2], x[3])] = v;
        dirty_ = true;
    }
    const std::vector<double> &tmat() const { return h_; }
    const std::vector<double> &eri() const { return eri_; }
    // The device copy, (re)created after the integrals changed.
    cigpu_ham *device() {
        if (!dev_ || dirty_) {
            cigpu_ham *h = nullptr;
            check(cigpu_ham_create(L_, nup_, ndown_, econst_, h_.data(), eri_.data(), &h), "cigpu_ham_create");
            dev_.reset(h);
            dirty_ = false;
        }
        return dev_.get();
    }

   private:
    size_t idx(int p, int q, int r, int s) const { return (((size_t)p * L_ + q) * L_ + r) * L_ + s; }
    struct Del {
        void operator()(cigpu_ham *h) const { cigpu_ham_destroy(h); }
    };
    int L_, nup_, ndown_;
    double econst_;
    double hf_energy_ = 0;
    std::vector<double> h_, eri_;
    std::unique_ptr<cigpu_ham, Del> dev_;
    bool dirty_ = true;
};

class SparseMatrix_CRS_Sym {
   public:
    explicit SparseMatrix_CRS_Sym(cigpu_crs *c) : crs_(c) {
        check(cigpu_crs_dims(c, &n_, &nnz_upper_, &nnz_full_), "cigpu_crs_dims");
    }
    int getn() const { return (int)n_; }
    int getm() const { return (int)n_; }
    int datasize() const { return (int)nnz_upper_; }
    int64_t nnz_full() const { return nnz_full_; }
    // y = H x with host buffers (SparseMatrix_CRS_Sym::mvprod, SparseMatrix_CRS.cpp:700-723)
    void mvprod(const double *x, double *y) const { check(cigpu_mvprod(crs_.get(), x, y, nullptr), "cigpu_mvprod"); }
    // Element (i, j) of the symmetric matrix (SparseMatrix_CRS_Sym::operator()).
    double operator()(unsigned i, unsigned j) const {
        if (i > j) std::swap(i, j);
        upper();
        for (uint32_t k = row_[i]; k < row_[i + 1]; ++k)
            if (col_[k] == j) return data_[k];
        return 0.0;
    }
    // The reference arrays data/col/row (SparseMatrix_CRS.h:107-111), exported once.
    const std::vector<uint32_t> &row() const { return (upper(), row_); }
    const std::vector<uint32_t> &col() const { return (upper(), col_); }
    const std::vector<double> &data() const { return (upper(), data_); }
    cigpu_crs *handle() const { return crs_.get(); }

   private:
    void upper() const {
        if (!row_.empty()) return;
        row_.resize(n_ + 1);
        col_.resize(nnz_upper_);
        data_.resize(nnz_upper_);
        check(cigpu_crs_export_upper(crs_.get(), row_.data(), col_.data(), data_.data()), "cigpu_crs_export_upper");
    }
    struct Del {
        void operator()(cigpu_crs *c) const { cigpu_crs_destroy(c); }
    };
    std::unique_ptr<cigpu_crs, Del> crs_;
    int64_t n_ = 0, nnz_upper_ = 0, nnz_full_ = 0;
    mutable std::vector<uint32_t> row_, col_;
    mutable std::vector<double> data_;
};

class CIMethod;

class CIDens {
   public:
    explicit CIDens(CIMethod *cim, unsigned state = 0) : cim_(cim), state_(state) {}
    virtual ~CIDens() = default;
    void construct_density(bool twordm = true);
    unsigned dim() const;
    double get_one_rdm(int spin, int orb1, int orb2) const {
        const int L = (int)dim();
        return one_[((size_t)spin * L + orb1) * L + orb2];
    }
    // CIDens::get_two_rdm (CIDens.cpp:166-190): spin 0 = aa, 1 = ab, 2 = bb
    double get_two_rdm(int spin, int i, int j, int k, int l) const {
        const int L = (int)dim();
        if (spin == 1) return ab_[((size_t)i * L + j) * L * L + (size_t)k * L + l];
        if (i == j || k == l) return 0.0;
        double sign = 1.0;
        if (i > j) { std::swap(i, j); sign = -sign; }
        if (k > l) { std::swap(k, l); sign = -sign; }
        const int np = L * (L - 1) / 2;
        const size_t a = (size_t)(i * L + j - (i + 1) * (i + 2) / 2), b = (size_t)(k * L + l - (k + 1) * (k + 2) / 2);
        return sign * (spin == 0 ? aa_ : bb_)[a * np + b];
    }
    double get_one_electron_energy() const;
    double get_two_electron_energy() const;
    double get_dens_energy() const;
    // CIDens::test_invariants (CIDens.cpp:365-409), throwing instead of exiting.
    void test_invariants(bool twordm = true) const;
    std::pair<bool, bool> is_constructed() const { return solved_; }

   protected:
    friend class CIMethod;
    CIMethod *cim_;
    unsigned state_;
    std::pair<bool, bool> solved_{false, false};
    std::vector<double> one_, aa_, ab_, bb_;
};

class DensFCI : public CIDens {
   public:
    using CIDens::CIDens;
};
class DensDOCI : public CIDens {
   public:
    using CIDens::CIDens;
};
class DensFILE : public CIDens {
   public:
    using CIDens::CIDens;
};

class CIMethod {
   public:
    CIMethod(Hamiltonian *ham, int method, int precision) : ham_(ham), method_(method), precision_(precision) {}
    virtual ~CIMethod() = default;
    virtual int get_dim() = 0;
    virtual std::string get_name() = 0;
    virtual std::unique_ptr<CIDens> get_density() = 0;

    virtual void build_ci() {
        cigpu_crs *c = nullptr;
        check(cigpu_build(ham_->device(), method_, precision_, nullptr, &c), "cigpu_build");
        mat_.reset(new SparseMatrix_CRS_Sym(c));
    }
    // CIMethod::solve (CIMethod.cpp:241-264): lowest eigenpair only.
    virtual void solve(int neigval = 1) {
        if (neigval != 1) throw Error(CIGPU_ENOTSUP, "solve: lowest eigenpair only");
        if (!mat_) build_ci();
        eigvec_.assign((size_t)get_dim(), 0.0);
        const int st = cigpu_solve(mat_->handle(), tol_, 0, nullptr, eigvec_.data(), &info_);
        if (st != CIGPU_OK && st != CIGPU_ENOCONV) check(st, "cigpu_solve");
        eigval_ = info_.e0 - ham_->getEconst();
        solved_ = true;
        cid_.reset();
    }
    double get_ci_energy(int neigval = 0) const {
        (void)neigval;
        return eigval_ + ham_->getEconst();
    }
    double get_eigvec(int numstate, int numvec) const {
        (void)numvec;
        return eigvec_[(size_t)numstate];
    }
    std::vector<double> get_eigvec(int numvec) const {
        (void)numvec;
        return eigvec_;
    }
    // CIMethod::set_ham (CIMethod.cpp:117-126)
    void set_ham(Hamiltonian *ham, bool build = true) {
        ham_ = ham;
        mat_.reset();
        solved_ = false;
        cid_.reset();
        if (build) build_ci();
    }
    void construct_density(unsigned state = 0, bool trdm = true) {
        if (state != 0) throw Error(CIGPU_ENOTSUP, "construct_density: ground state only");
        if (!cid_) cid_ = get_density();
        if (!cid_->is_constructed().first || (trdm && !cid_->is_constructed().second)) cid_->construct_density(trdm);
    }
    CIDens *density() { return cid_.get(); }
    int get_method() const { return method_; }
    int get_precision() const { return precision_; }
    double get_tolerance() const { return tol_; }
    // The CI-vector block of the reference's output (Output.cpp:135-263).
    virtual void print_ci_vec(const std::string &path, double nauw = -1.0) {
        check(cigpu_write_civec(path.c_str(), method_, get_l(), gNup(), gNdown(), (int64_t)eigvec_.size(),
                                eigvec_.data(), get_ci_energy(), get_econst(), nauw, nullptr, nullptr, 1, nullptr),
              "cigpu_write_civec");
    }
    // CIMethod::print_one_rdm / print_two_rdm (CIMethod.cpp:184-195) into a file.
    void print_rdm(const std::string &path, bool trdm = true);
    Hamiltonian *get_ham() { return ham_; }
    SparseMatrix_CRS_Sym &get_mat() {
        if (!mat_) build_ci();
        return *mat_;
    }
    int gNup() const { return ham_->getnup(); }
    int gNdown() const { return ham_->getndown(); }
    int get_l() const { return ham_->getL(); }
    double get_econst() const { return ham_->getEconst(); }
    bool is_solved() const { return solved_; }
    void set_tolerance(double tol) { tol_ = tol; }
    const cigpu_solve_info &solve_info() const { return info_; }

   protected:
    Hamiltonian *ham_;
    int method_, precision_;
    double tol_ = 1e-8;
    std::unique_ptr<SparseMatrix_CRS_Sym> mat_;
    std::vector<double> eigvec_;
    double eigval_ = 0;
    bool solved_ = false;
    cigpu_solve_info info_{};
    std::unique_ptr<CIDens> cid_;
};

class FCI : public CIMethod {
   public:
    explicit FCI(Hamiltonian *ham, int precision = CIGPU_FP64) : CIMethod(ham, CIGPU_FCI, precision) { build_ci(); }
    int get_dim() override { return (int)(binomial(ham_->getL(), ham_->getnup()) * binomial(ham_->getL(), ham_->getndown())); }
    std::string get_name() override { return "FCI"; }
    std::unique_ptr<CIDens> get_density() override { return std::unique_ptr<CIDens>(new DensFCI(this)); }
    int gUpDim() const { return (int)binomial(ham_->getL(), ham_->getnup()); }
    int gDownDim() const { return (int)binomial(ham_->getL(), ham_->getndown()); }
};

class DOCI : public CIMethod {
   public:
    explicit DOCI(Hamiltonian *ham, int precision = CIGPU_FP64) : CIMethod(ham, CIGPU_DOCI, precision) { build_ci(); }
    int get_dim() override { return (int)binomial(ham_->getL(), ham_->getnup()); }
    std::string get_name() override { return "DOCI"; }
    std::unique_ptr<CIDens> get_density() override { return std::unique_ptr<CIDens>(new DensDOCI(this)); }
};

// FCI_File / CI_Big (CIMethod.h:164-189): CI over the determinant list of a file
// (Permutator_File format) in list order; CI_Big keeps no matrix (every matvec
// recomputes the elements).
class FCI_File : public CIMethod {
   public:
    FCI_File(Hamiltonian *ham, const std::string &permfile, int precision = CIGPU_FP64)
        : CIMethod(ham, CIGPU_DETS, precision), permfile_(permfile) {
        words_ = ham->getL() <= 64 ? 1 : 2;
        int64_t n = 0;
        int nb = 0;
        check(cigpu_dets_read(permfile.c_str(), words_, 0, nullptr, nullptr, &n, &nb), "cigpu_dets_read");
        up_.resize((size_t)n * words_);
        down_.resize((size_t)n * words_);
        check(cigpu_dets_read(permfile.c_str(), words_, n, up_.data(), down_.data(), &n, &nb), "cigpu_dets_read");
        build_ci();
    }
    void build_ci() override {
        cigpu_crs *c = nullptr;
        check(cigpu_build_dets(ham_->device(), get_dim(), words_, up_.data(), down_.data(), storage(), precision_,
                               nullptr, &c),
              "cigpu_build_dets");
        mat_.reset(new SparseMatrix_CRS_Sym(c));
    }
    int get_dim() override { return (int)(up_.size() / words_); }
    std::string get_name() override { return "FCI_File"; }
    std::unique_ptr<CIDens> get_density() override { return std::unique_ptr<CIDens>(new DensFILE(this)); }
    // Permutator::get_clean_detfile (Permutator.cpp:88-100)
    std::string get_clean_detfile() const {
        std::string f = permfile_.substr(permfile_.find_last_of("/\\") + 1);
        f = f.substr(0, f.find_last_of('.'));
        std::string out;
        for (char ch : f)
            if (std::string("_()-./\\").find(ch) == std::string::npos) out += ch;
        return out;
    }
    void print_ci_vec(const std::string &path, double nauw = -1.0) override {
        const std::string name = get_clean_detfile();
        check(cigpu_write_civec(path.c_str(), CIGPU_DETS, get_l(), gNup(), gNdown(), (int64_t)eigvec_.size(),
                                eigvec_.data(), get_ci_energy(), get_econst(), nauw, up_.data(), down_.data(), words_,
                                name.c_str()),
              "cigpu_write_civec");
    }

   protected:
    virtual int storage() const { return CIGPU_DETS_CRS; }
    std::string permfile_;
    int words_ = 1;
    std::vector<uint64_t> up_, down_;
};

class CI_Big : public FCI_File {
   public:
    CI_Big(Hamiltonian *ham, const std::string &permfile) : FCI_File(ham, permfile, CIGPU_FP64) {}
    std::string get_name() override { return "CI_Big"; }

   protected:
    int storage() const override { return CIGPU_DETS_ONTHEFLY; }
};

// ---- orbital optimisers (SimulatedAnnealing.cpp, LocalMinimizer.cpp) over cigpu_orbopt ----
// The optimiser owns the rotated Hamiltonians (as OrbitalOptimization owns _optham);
// update_cim() hands the current one to the CIMethod and solves it there.
class OrbitalOptimization {
   public:
    explicit OrbitalOptimization(CIMethod *cim, uint64_t seed = 0) : cim_(cim) {
        if (!cim->is_solved()) cim->solve();
        cigpu_orbopt_config cfg{};
        cfg.method = cim->get_method();
        cfg.precision = cim->get_precision();
        cfg.tol = cim->get_tolerance();
        cfg.warm_start = 1;
        cfg.seed = seed;
        cigpu_orbopt *o = nullptr;
        check(cigpu_orbopt_create(cim->get_ham()->device(), &cfg, &o), "cigpu_orbopt_create");
        opt_.reset(o);
    }
    virtual ~OrbitalOptimization() = default;
    double get_opt_ci_energy() const { return stats().e_opt; }
    std::vector<double> get_opt_unitary() const {
        std::vector<double> u((size_t)cim_->get_l() * cim_->get_l());
        check(cigpu_orbopt_get(opt_.get(), nullptr, u.data(), nullptr, nullptr), "cigpu_orbopt_get");
        return u;
    }
    cigpu_orbopt_stats stats() const {
        cigpu_orbopt_stats st{};
        check(cigpu_orbopt_get(opt_.get(), nullptr, nullptr, nullptr, &st), "cigpu_orbopt_get");
        return st;
    }
    // OrbitalOptimization::update_cim (SimulatedAnnealing.cpp:83-87)
    void update_cim() {
        cigpu_ham *h = nullptr;
        check(cigpu_orbopt_ham(opt_.get(), &h), "cigpu_orbopt_ham");
        Hamiltonian *ham = cim_->get_ham();
        optham_.reset(new Hamiltonian(h, ham->getL(), ham->getnup(), ham->getndown(), ham->getEconst()));
        cim_->set_ham(optham_.get());
        cim_->solve();
    }
    // set_cim_optimal (SimulatedAnnealing.cpp:69-74)
    void set_cim_optimal() {
        check(cigpu_orbopt_set_optimal(opt_.get()), "cigpu_orbopt_set_optimal");
        update_cim();
    }
    double get_cim_no() {
        double e = 0;
        check(cigpu_orbopt_natural(opt_.get(), cim_->get_method(), &e), "cigpu_orbopt_natural");
        return e;
    }
    double get_fci_no() {
        double e = 0;
        check(cigpu_orbopt_natural(opt_.get(), CIGPU_FCI, &e), "cigpu_orbopt_natural");
        return e;
    }

   protected:
    struct Del {
        void operator()(cigpu_orbopt *o) const { cigpu_orbopt_destroy(o); }
    };
    CIMethod *cim_;
    std::unique_ptr<cigpu_orbopt, Del> opt_;
    std::unique_ptr<Hamiltonian> optham_;
};

class SimulatedAnnealing : public OrbitalOptimization {
   public:
    SimulatedAnnealing(CIMethod *cim, double temp, double change_temp, double angle, double change_angle,
                       uint64_t seed = 0)
        : OrbitalOptimization(cim, seed) {
        p_.temp = temp;
        p_.change_temp = change_temp;
        p_.max_angle = angle;
        p_.change_angle = change_angle;
        p_.steps = 20000;
        p_.max_unaccept = 2000;
        p_.min_angle = 1e-7;
        p_.speculate = 1;
    }
    void set_steps(int64_t steps) { p_.steps = steps; }
    void set_speculate(int k) { p_.speculate = k; }
    // SimulatedAnnealing::optimize (SimulatedAnnealing.cpp:306-391)
    double optimize() {
        double e = 0;
        check(cigpu_orbopt_anneal(opt_.get(), &p_, &e), "cigpu_orbopt_anneal");
        update_cim();
        return e;
    }

   private:
    cigpu_anneal_params p_{};
};

class LocalMinimizer : public OrbitalOptimization {
   public:
    explicit LocalMinimizer(CIMethod *cim, uint64_t seed = 0) : OrbitalOptimization(cim, seed) {
        if (cim->get_method() != CIGPU_DOCI) throw Error(CIGPU_ENOTSUP, "LocalMinimizer: DOCI only");
        p_.conv_crit = 1e-6;
        p_.conv_steps = 25;
        p_.max_iters = 1000;
    }
    void set_conv_crit(double crit) { p_.conv_crit = crit; }
    void set_conv_steps(int steps) { p_.conv_steps = steps; }
    double get_conv_crit() const { return p_.conv_crit; }
    // LocalMinimizer::optimize (LocalMinimizer.cpp:130-235)
    double optimize(bool dist_choice = false) {
        p_.dist_choice = dist_choice ? 1 : 0;
        double e = 0;
        check(cigpu_orbopt_local(opt_.get(), &p_, &e), "cigpu_orbopt_local");
        update_cim();
        return e;
    }

   private:
    cigpu_local_params p_{};
};

// ---- CIDens members that need CIMethod ----
inline unsigned CIDens::dim() const { return (unsigned)cim_->get_l(); }

inline void CIDens::construct_density(bool twordm) {
    const int L = (int)dim(), np = L * (L - 1) / 2;
    one_.assign((size_t)2 * L * L, 0.0);
    aa_.assign(twordm ? (size_t)np * np : 0, 0.0);
    bb_.assign(twordm ? (size_t)np * np : 0, 0.0);
    ab_.assign(twordm ? (size_t)L * L * L * L : 0, 0.0);
    const std::vector<double> c = cim_->get_eigvec(0);
    check(cigpu_rdm(cim_->get_mat().handle(), c.data(), one_.data(), twordm ? aa_.data() : nullptr,
                    twordm ? ab_.data() : nullptr, twordm ? bb_.data() : nullptr),
          "cigpu_rdm");
    solved_ = {true, twordm};
}

inline void CIMethod::print_rdm(const std::string &path, bool trdm) {
    construct_density(0, trdm);
    const CIDens &d = *cid_;
    check(cigpu_write_rdm(path.c_str(), get_l(), d.one_.data(), trdm ? d.aa_.data() : nullptr,
                          trdm ? d.ab_.data() : nullptr, trdm ? d.bb_.data() : nullptr),
          "cigpu_write_rdm");
}

inline double CIDens::get_one_electron_energy() const {
    const int L = (int)dim();
    double e = 0;
    for (int i = 0; i < L; ++i)
        for (int j = 0; j < L; ++j)
            e += cim_->get_ham()->getTmat(i, j) * (get_one_rdm(0, i, j) + get_one_rdm(1, i, j));
    return e;
}

inline double CIDens::get_two_electron_energy() const {
    const int L = (int)dim();
    double e = 0;
    for (int i = 0; i < L; ++i)
        for (int j = 0; j < L; ++j)
            for (int k = 0; k < L; ++k)
                for (int l = 0; l < L; ++l) {
                    const double v = cim_->get_ham()->getVmat(i, j, k, l);
                    e += v * get_two_rdm(0, i, j, k, l) + 2 * v * get_two_rdm(1, i, j, k, l) +
                         v * get_two_rdm(2, i, j, k, l);
                }
    return 0.5 * e;
}

inline double CIDens::get_dens_energy() const {
    return get_one_electron_energy() + get_two_electron_energy() + cim_->get_econst();
}

inline void CIDens::test_invariants(bool twordm) const {
    const int L = (int)dim(), N = cim_->gNup() + cim_->gNdown();
    double tr = 0;
    for (int s = 0; s < 2; ++s)
        for (int i = 0; i < L; ++i) tr += get_one_rdm(s, i, i);
    if (std::fabs(tr - N) > 1e-9) throw Error(CIGPU_EINVAL, "trace of the 1-RDM differs from N");
    if (!twordm) return;
    double t2 = 0;
    for (int i = 0; i < L; ++i) {
        for (int j = 0; j < L; ++j) t2 += get_two_rdm(1, i, j, i, j);
        for (int j = i + 1; j < L; ++j) t2 += get_two_rdm(0, i, j, i, j) + get_two_rdm(2, i, j, i, j);
    }
    if (std::fabs(t2 - 0.5 * N * (N - 1)) > 1e-5) throw Error(CIGPU_EINVAL, "trace of the 2-RDM differs from N(N-1)/2");
}

}  // namespace ciflow_gb300
