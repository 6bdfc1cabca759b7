// On-disk formats of the path (host code): the psi4 integral text dump that
// Hamiltonian reads and writes (Hamiltonian.cpp:646-885), and the text dumps of a
// CI vector (Output.cpp:124-133, 190-263) and of the RDMs (CIDens.cpp:978-1026,
// CIMethod.cpp:184-195).
//
// Numbers are written with C's "%.16g" (what an ostream with precision 16 prints)
// where the reference uses precision 16; the integral dump uses "%.17g" so that a
// file round-trips every double exactly (the reference writes 15 digits).
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "../../include/cigpu.h"

namespace {

constexpr int kMaxOrbitals = 128;

// The reference takes "<label> = <value> " and parses line.substr(pos + 2, size - pos - 3):
// the text after "= " without the line's last character.
std::string after_equals(const std::string &line) {
    const size_t pos = line.find('=');
    if (pos == std::string::npos || pos + 2 > line.size()) return std::string();
    const size_t len = line.size() >= pos + 3 ? line.size() - pos - 3 : 0;
    return line.substr(pos + 2, len);
}

// "i j value " lines: fields separated by single spaces; the value is the text after
// the last index without the line's last character (Hamiltonian.cpp:801-846).
bool parse_indices(const std::string &line, int nidx, int *idx, double *value) {
    size_t pos = 0;
    for (int k = 0; k < nidx; ++k) {
        const size_t p2 = line.find(' ', pos);
        if (p2 == std::string::npos) return false;
        char *end = nullptr;
        const std::string f = line.substr(pos, p2 - pos);
        const long v = std::strtol(f.c_str(), &end, 10);
        if (f.empty() || *end != '\0') return false;
        idx[k] = (int)v;
        pos = p2 + 1;
    }
    if (line.size() < pos + 1) return false;
    const std::string f = line.substr(pos, line.size() - pos - 1);
    char *end = nullptr;
    *value = std::strtod(f.c_str(), &end);
    return end != f.c_str();
}

void write_g(FILE *f, double v, int digits) { std::fprintf(f, "%.*g", digits, v); }

std::string bits(const uint64_t *s, int L) {
    std::string out((size_t)L, '0');
    for (int o = 0; o < L; ++o)
        if ((s[o >> 6] >> (o & 63)) & 1) out[(size_t)(L - 1 - o)] = '1';
    return out;
}

}  // namespace

extern "C" {

int cigpu_ham_read_psi4(const char *path, int *L, int *nup, int *ndown, double *econst, double *h, double *eri,
                        int *irreps, double *hf_energy) {
    if (!path || !L || !nup || !ndown || !econst) return CIGPU_EINVAL;
    std::ifstream in(path);
    if (!in.is_open()) return CIGPU_ENOTFOUND;
    std::string line;
    // wind to the start of the dump
    bool found = false;
    while (std::getline(in, line))
        if (line.find("****  Molecular Integrals") != std::string::npos) {
            found = true;
            break;
        }
    if (!found) return CIGPU_EINVAL;
    std::string hdr[7];
    for (int k = 0; k < 7; ++k)
        if (!std::getline(in, hdr[k])) return CIGPU_EINVAL;
    // Nalpha, Nbeta, Symmetry Label, Nirreps, Nuclear Repulsion Energy, Number Of MOs, "Irreps Of ..."
    *nup = std::atoi(after_equals(hdr[0]).c_str());
    *ndown = std::atoi(after_equals(hdr[1]).c_str());
    *econst = std::atof(after_equals(hdr[4]).c_str());
    *L = std::atoi(after_equals(hdr[5]).c_str());
    const int n = *L;
    if (n < 1 || n > kMaxOrbitals || *nup < 0 || *ndown < 0 || *nup > n || *ndown > n) return CIGPU_EINVAL;
    std::string irr;
    if (!std::getline(in, irr)) return CIGPU_EINVAL;
    if (irreps) {
        // one digit per orbital at even positions (Hamiltonian.cpp:779-783)
        for (int k = 0; k < n; ++k) irreps[k] = (size_t)(2 * k) < irr.size() ? irr[(size_t)(2 * k)] - '0' : 0;
    }
    if (!h && !eri) return CIGPU_OK;  // header only
    // optional overlap / unitary sections are skipped: wind to the first "**" line
    found = false;
    while (std::getline(in, line))
        if (line.compare(0, 2, "**") == 0) {
            found = true;
            break;
        }
    if (!found) return CIGPU_EINVAL;
    const size_t L1 = n, L2 = L1 * L1, L3 = L2 * L1;
    if (h) std::memset(h, 0, sizeof(double) * L2);
    if (eri) std::memset(eri, 0, sizeof(double) * L2 * L2);
    // one-electron integrals until a line starting with '*': setTmat(i, j) sets both triangles
    while (std::getline(in, line) && line.compare(0, 1, "*") != 0) {
        int ij[2];
        double v = 0;
        if (!parse_indices(line, 2, ij, &v)) return CIGPU_EINVAL;
        if (ij[0] < 0 || ij[1] < 0 || ij[0] >= n || ij[1] >= n) return CIGPU_EINVAL;
        if (h) h[ij[0] * L1 + ij[1]] = h[ij[1] * L1 + ij[0]] = v;
    }
    // two-electron integrals in chemist order (pq|rs): every permutation partner is set
    while (std::getline(in, line) && line.compare(0, 1, "*") != 0) {
        int q4[4];
        double v = 0;
        if (!parse_indices(line, 4, q4, &v)) return CIGPU_EINVAL;
        for (int k = 0; k < 4; ++k)
            if (q4[k] < 0 || q4[k] >= n) return CIGPU_EINVAL;
        if (eri) {
            const int p = q4[0], q = q4[1], r = q4[2], s = q4[3];
            const int perm[8][4] = {{p, q, r, s}, {q, p, r, s}, {p, q, s, r}, {q, p, s, r},
                                    {r, s, p, q}, {s, r, p, q}, {r, s, q, p}, {s, r, q, p}};
            for (const auto &t : perm) eri[t[0] * L3 + t[1] * L2 + t[2] * L1 + t[3]] = v;
        }
    }
    if (hf_energy) *hf_energy = std::atof(after_equals(line).c_str());
    return CIGPU_OK;
}

int cigpu_ham_write_psi4(const char *path, int L, int nup, int ndown, double econst, const double *h,
                         const double *eri, double hf_energy) {
    if (!path || !h || !eri || L < 1 || L > kMaxOrbitals || nup < 0 || ndown < 0) return CIGPU_EINVAL;
    FILE *f = std::fopen(path, "w");
    if (!f) return CIGPU_ENOTFOUND;
    const size_t L1 = L, L2 = L1 * L1, L3 = L2 * L1;
    std::fprintf(f, "****  Molecular Integrals Start Here \n");
    std::fprintf(f, "Nalpha = %d \nNbeta = %d \nSymmetry Label = c1 \nNirreps = 1 \n", nup, ndown);
    std::fprintf(f, "Nuclear Repulsion Energy = ");
    write_g(f, econst, 17);
    std::fprintf(f, " \nNumber Of Molecular Orbitals = %d \nIrreps Of Molecular Orbitals = \n", L);
    for (int i = 0; i < L; ++i) std::fprintf(f, "0 ");
    std::fprintf(f, "\nDOCC =  \nSOCC =  \n#### There is no overlap.   \n****  MO OEI \n");
    for (int i = 0; i < L; ++i)
        for (int j = 0; j < L; ++j)
            if (h[i * L1 + j] != 0.) {
                std::fprintf(f, "%d %d ", i, j);
                write_g(f, h[i * L1 + j], 17);
                std::fprintf(f, " \n");
            }
    std::fprintf(f, "****  MO TEI \n");
    // canonical elements (p >= q, r >= s, pq >= rs); the reader sets all partners
    for (int p = 0; p < L; ++p)
        for (int q = 0; q <= p; ++q)
            for (int r = 0; r <= p; ++r)
                for (int s = 0; s <= r; ++s) {
                    if (p * L + q < r * L + s) continue;
                    const double v = eri[p * L3 + q * L2 + r * L1 + s];
                    if (v == 0.) continue;
                    std::fprintf(f, "%d %d %d %d ", p, q, r, s);
                    write_g(f, v, 17);
                    std::fprintf(f, " \n");
                }
    std::fprintf(f, "****  HF Energy = ");
    write_g(f, hf_energy, 17);
    std::fprintf(f, " \n****  Molecular Integrals End Here \n\n");
    const bool ok = std::ferror(f) == 0;
    std::fclose(f);
    return ok ? CIGPU_OK : CIGPU_EINVAL;
}

int cigpu_write_civec(const char *path, int method, int L, int nup, int ndown, int64_t dim, const double *c,
                      double e0, double econst, double threshold, const uint64_t *up, const uint64_t *down, int words,
                      const char *list_name) {
    if (!path || !c || dim < 1 || L < 1 || L > kMaxOrbitals) return CIGPU_EINVAL;
    if (method == CIGPU_DETS && (!up || !down || (words != 1 && words != 2) || (L > 64 && words < 2)))
        return CIGPU_EINVAL;
    if ((method == CIGPU_FCI || method == CIGPU_DOCI) && L > 63) return CIGPU_EINVAL;
    FILE *f = std::fopen(path, "w");
    if (!f) return CIGPU_ENOTFOUND;
    // OutputSingleFile::print_solutions (Output.cpp:135-144)
    std::fprintf(f, "#the obtained energy spectrum with the nuclear repulsion energy (");
    write_g(f, econst, 6);
    std::fprintf(f, ") added is: \n#energies: \n");
    write_g(f, e0, 16);
    std::fprintf(f, "\n");
    int64_t count = 0;
    auto entry2 = [&](int64_t idx, const uint64_t *u, const uint64_t *d, double v) {
        std::fprintf(f, "%lld\t%s\t%s\t", (long long)idx, bits(u, L).c_str(), bits(d, L).c_str());
        write_g(f, v, 16);
        std::fprintf(f, "\n");
    };
    if (method == CIGPU_FCI) {
        // OutputSFFCI::print_ci_vec (Output.cpp:216-241): alpha-major, colex strings
        std::fprintf(f, "#CIMETHOD= FCI\n#Start  FCI vec 0 only significant determinants are kept (abs(coef) > ");
        write_g(f, threshold, 16);
        std::fprintf(f, " )\n#dimension FCI is: %lld\n#index\tupbitstring\tdownbitstring\tfci_coef\n", (long long)dim);
        std::vector<uint64_t> ua, db;
        for (uint64_t s = nup ? (((uint64_t)1 << nup) - 1) : 0;; ) {
            ua.push_back(s);
            if (nup == 0 || nup == L) break;
            const uint64_t t = s | (s - 1);
            const uint64_t nx = (t + 1) | (((~t & (t + 1)) - 1) >> (__builtin_ctzll(s) + 1));
            if (nx >> L) break;
            s = nx;
        }
        for (uint64_t s = ndown ? (((uint64_t)1 << ndown) - 1) : 0;; ) {
            db.push_back(s);
            if (ndown == 0 || ndown == L) break;
            const uint64_t t = s | (s - 1);
            const uint64_t nx = (t + 1) | (((~t & (t + 1)) - 1) >> (__builtin_ctzll(s) + 1));
            if (nx >> L) break;
            s = nx;
        }
        if ((int64_t)(ua.size() * db.size()) != dim) {
            std::fclose(f);
            return CIGPU_EINVAL;
        }
        int64_t idx = 0;
        for (size_t a = 0; a < ua.size(); ++a)
            for (size_t b = 0; b < db.size(); ++b, ++idx)
                if (std::fabs(c[idx]) >= threshold) {
                    entry2(idx, &ua[a], &db[b], c[idx]);
                    ++count;
                }
        std::fprintf(f, "#Significant determinants: %lld of %lld\n#End vecoutput\n", (long long)count, (long long)dim);
    } else if (method == CIGPU_DOCI) {
        // OutputSFDOCI::print_ci_vec (Output.cpp:190-210), every index with its own pair string
        std::fprintf(f, "#CIMETHOD=  DOCI\n#Start  DOCI vec 0 only significant determinants are kept (abs(coef) > ");
        write_g(f, threshold, 16);
        std::fprintf(f, " )\n#dimension DOCI  is: %lld\n#index\tupbitstring\tdoci_coef\n", (long long)dim);
        uint64_t s = nup ? (((uint64_t)1 << nup) - 1) : 0;
        for (int64_t idx = 0; idx < dim; ++idx) {
            if (std::fabs(c[idx]) >= threshold) {
                std::fprintf(f, "%lld\t%s\t", (long long)idx, bits(&s, L).c_str());
                write_g(f, c[idx], 16);
                std::fprintf(f, "\n");
                ++count;
            }
            if (nup > 0 && nup < L) {
                const uint64_t t = s | (s - 1);
                s = (t + 1) | (((~t & (t + 1)) - 1) >> (__builtin_ctzll(s) + 1));
            }
        }
        std::fprintf(f, "#Significant determinants: %lld\n#End vecoutput\n", (long long)count);
    } else if (method == CIGPU_DETS) {
        // OutputSFFCI_File::print_ci_vec (Output.cpp:247-263): the list order
        std::fprintf(f, "#CIMETHOD= configuration interaction of all the determinants in %s\n",
                     list_name ? list_name : "the list");
        std::fprintf(f, "#Start  FCI_File vec 0 only significant determinants are kept (abs(coef) > ");
        write_g(f, threshold, 16);
        std::fprintf(f, " )\n#CI dimension in file is: %lld\n#index\tupbitstring\tdownbitstring\tfci_coef\n",
                     (long long)dim);
        for (int64_t idx = 0; idx < dim; ++idx)
            if (std::fabs(c[idx]) >= threshold) {
                entry2(idx, up + idx * words, down + idx * words, c[idx]);
                ++count;
            }
        std::fprintf(f, "#Significant determinants: %lld of %lld\n#End vecoutput\n", (long long)count, (long long)dim);
    } else {
        std::fclose(f);
        return CIGPU_EINVAL;
    }
    const bool ok = std::ferror(f) == 0;
    std::fclose(f);
    return ok ? CIGPU_OK : CIGPU_EINVAL;
}

int cigpu_write_rdm(const char *path, int L, const double *rdm1, const double *rdm2_aa, const double *rdm2_ab,
                    const double *rdm2_bb) {
    if (!path || !rdm1 || L < 1 || L > 64) return CIGPU_EINVAL;
    const bool two = rdm2_aa && rdm2_ab && rdm2_bb;
    FILE *f = std::fopen(path, "w");
    if (!f) return CIGPU_ENOTFOUND;
    const size_t L1 = L, L2 = L1 * L1, np = L1 * (L1 - 1) / 2;
    // CIMethod::print_one_rdm + CIDens::print_one_dens (CIMethod.cpp:184-189, CIDens.cpp:978-994)
    std::fprintf(f, "#The eigenstate from which the density matrix is constructed: 0\n#THE 1RDM:\n");
    for (int sp = 0; sp < 2; ++sp) {
        std::fprintf(f, "#One rdm of the %d spin electrons.\n", sp);
        int count = 0;
        for (int i = 0; i < L; ++i)
            for (int k = i; k < L; ++k) {
                const double v = rdm1[sp * L2 + i * L1 + k];
                if (std::fabs(v) >= 1e-12) {
                    std::fprintf(f, "%d %d ", i, k);
                    write_g(f, v, 16);
                    std::fprintf(f, "\n");
                    ++count;
                }
            }
        std::fprintf(f, "#We obtained %d non zero elements.\n", count);
    }
    if (two) {
        // CIMethod::print_two_rdm + CIDens::print_two_dens (CIMethod.cpp:191-195, CIDens.cpp:996-1026)
        std::fprintf(f, "#THE 2RDM:\n");
        auto pidx = [&](int p, int q) { return (size_t)(p * L + q - (p + 1) * (p + 2) / 2); };
        auto g = [&](int sp, int i, int k, int l, int m) {
            if (sp == 1) return rdm2_ab[(size_t)(i * L + k) * L2 + (size_t)(l * L + m)];
            const double *X = sp == 0 ? rdm2_aa : rdm2_bb;
            return X[pidx(i, k) * np + pidx(l, m)];  // i < k and l < m in these loops
        };
        for (int sp = 0; sp < 3; ++sp) {
            std::fprintf(f, "#Two rdm case : %d---------------------------------------------\n", sp);
            int count = 0;
            for (int i = 0; i < L; ++i)
                for (int k = sp == 1 ? 0 : i + 1; k < L; ++k)
                    for (int l = 0; l < L; ++l)
                        for (int m = sp == 1 ? 0 : l + 1; m < L; ++m) {
                            const double v = g(sp, i, k, l, m);
                            if (std::fabs(v) > 1e-12) {
                                std::fprintf(f, "%d %d %d %d ", i, k, l, m);
                                write_g(f, v, 16);
                                std::fprintf(f, "\n");
                                ++count;
                            }
                        }
            std::fprintf(f, "#We obtained %d non zero elements.\n", count);
        }
    }
    const bool ok = std::ferror(f) == 0;
    std::fclose(f);
    return ok ? CIGPU_OK : CIGPU_EINVAL;
}

}  // extern "C"
