// deck_io.h -- particle decks of the CERN-F77 code and the GPU-C VTK output
// (host code of the library, no device work).
//
// Deck: in one directory, the real particles in f_xv.dat, f_state.dat and
// f_other.dat, the virtual (wall) particles in v_xv.dat, v_state.dat and
// v_other.dat (CERNsource/input.f:197-314 reads them, output.f:31-73 writes
// them):
//   *_xv.dat     line 1: the particle count; then per particle
//                "i x(1..dim) v(1..dim)"              format (1x, I6, 6(2x, e14.8))
//   *_state.dat  "i mass rho p u"                      format (1x, I6, 7(2x, e14.8))
//   *_other.dat  "i mat h"                             format (1x, I6, 2x, I4, 2x, e14.8)
// Indices run 1..np in the f_ files and np+1..np+nv in the v_ files. Reading
// is list-directed as in the Fortran (whitespace-separated, D or E exponents);
// writing reproduces the explicit formats character for character.
//
// VTK: the legacy ASCII unstructured grid of ArmandoThrust/armando.cu:1596-1670
// (points, one vertex cell per particle, material, density, pressure, energy,
// velocity).
#pragma once
#include <cctype>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace ag {
namespace deck {

// Fortran Ew.d with w = 14, d = 8: "0.dddddddd" and a two-digit exponent
// "E+xx" (three digits without the E beyond 99); the leading zero gives way to
// the sign of negative values.
inline std::string fortran_e14_8(double v) {
    char m[64];
    if (!std::isfinite(v)) return std::string(14, '*');
    int e10 = 0;
    std::string digits = "00000000";
    if (v != 0.0) {
        std::snprintf(m, sizeof m, "%.7e", std::fabs(v));  // d.ddddddde+XX: 8 significant digits
        digits.assign(1, m[0]);
        digits.append(m + 2, 7);
        e10 = std::atoi(std::strchr(m, 'e') + 1) + 1;  // 0.d1..d8 x 10^e10
    }
    std::string out = (v < 0.0) ? "-." : "0.";
    out += digits;
    char ex[16];
    const int a = e10 < 0 ? -e10 : e10;
    if (a <= 99) std::snprintf(ex, sizeof ex, "E%c%02d", e10 < 0 ? '-' : '+', a);
    else std::snprintf(ex, sizeof ex, "%c%03d", e10 < 0 ? '-' : '+', a);
    out += ex;
    if (out.size() > 14) return std::string(14, '*');
    return std::string(14 - out.size(), ' ') + out;
}

// Fortran Iw: right-justified, asterisks when it does not fit.
inline std::string fortran_i(long long v, int w) {
    char b[32];
    std::snprintf(b, sizeof b, "%lld", v);
    const std::string s(b);
    if ((int)s.size() > w) return std::string(w, '*');
    return std::string(w - s.size(), ' ') + s;
}

// List-directed number: E or D exponent, or a signed exponent without a
// letter ("0.12345678+100").
inline bool parse_real(const std::string& tok, double& out) {
    std::string t = tok;
    for (char& c : t)
        if (c == 'd' || c == 'D') c = 'E';
    size_t k = 1;
    for (; k < t.size(); ++k)
        if ((t[k] == '+' || t[k] == '-') && std::isdigit((unsigned char)t[k - 1])) {
            t.insert(k, 1, 'E');
            break;
        }
    char* end = nullptr;
    errno = 0;
    out = std::strtod(t.c_str(), &end);
    return end && *end == '\0' && !t.empty() && errno != ERANGE;
}

inline bool parse_int(const std::string& tok, long long& out) {
    char* end = nullptr;
    out = std::strtoll(tok.c_str(), &end, 10);
    return end && *end == '\0' && !tok.empty();
}

// Reads whitespace-separated tokens of a text file.
class Tokens {
public:
    explicit Tokens(const std::string& path) : f_(std::fopen(path.c_str(), "r")) {}
    ~Tokens() {
        if (f_) std::fclose(f_);
    }
    bool ok() const { return f_ != nullptr; }
    bool next(std::string& tok) {
        tok.clear();
        int c;
        while ((c = std::fgetc(f_)) != EOF && std::isspace(c)) {
        }
        if (c == EOF) return false;
        do {
            tok.push_back((char)c);
        } while ((c = std::fgetc(f_)) != EOF && !std::isspace(c));
        return true;
    }
    bool real(double& v) {
        std::string t;
        return next(t) && parse_real(t, v);
    }
    bool integer(long long& v) {
        std::string t;
        return next(t) && parse_int(t, v);
    }

private:
    FILE* f_;
};

inline std::string join(const std::string& dir, const char* name) {
    if (dir.empty()) return name;
    return (dir.back() == '/') ? dir + name : dir + "/" + name;
}

// Particle count on the first line of <prefix>_xv.dat; -1: no such file.
inline long long count(const std::string& dir, const char* prefix, std::string& err) {
    const std::string path = join(dir, (std::string(prefix) + "_xv.dat").c_str());
    Tokens t(path);
    if (!t.ok()) return -1;
    long long n = 0;
    if (!t.integer(n) || n < 0) {
        err = path + ": no particle count on the first line";
        return -2;
    }
    return n;
}

struct Arrays {
    float *x, *v, *mass, *rho, *p, *u, *h;
    int* itype;
};

// Reads particles [first, first + n) of the arrays from one prefix's files.
inline bool read_set(const std::string& dir, const char* prefix, int dim, long long first,
                     long long n, const Arrays& a, std::string& err) {
    const std::string pre(prefix);
    const std::string pxv = join(dir, (pre + "_xv.dat").c_str());
    const std::string pst = join(dir, (pre + "_state.dat").c_str());
    const std::string pot = join(dir, (pre + "_other.dat").c_str());
    Tokens xv(pxv), st(pst), ot(pot);
    if (!xv.ok() || !st.ok() || !ot.ok()) {
        err = "cannot open " + (!xv.ok() ? pxv : !st.ok() ? pst : pot);
        return false;
    }
    long long cnt = 0, im = 0, mat = 0;
    if (!xv.integer(cnt) || cnt != n) {
        err = pxv + ": particle count differs from the one given";
        return false;
    }
    double r[8];
    for (long long k = 0; k < n; ++k) {
        const long long i = first + k;
        bool good = xv.integer(im);
        for (int d = 0; d < 2 * dim && good; ++d) good = xv.real(r[d]);
        if (!good) {
            err = pxv + ": bad record " + std::to_string(k + 1);
            return false;
        }
        for (int d = 0; d < dim; ++d) {
            a.x[i * dim + d] = (float)r[d];
            a.v[i * dim + d] = (float)r[dim + d];
        }
        good = st.integer(im);
        for (int q = 0; q < 4 && good; ++q) good = st.real(r[q]);
        if (!good) {
            err = pst + ": bad record " + std::to_string(k + 1);
            return false;
        }
        a.mass[i] = (float)r[0];
        a.rho[i] = (float)r[1];
        a.p[i] = (float)r[2];
        a.u[i] = (float)r[3];
        if (!ot.integer(im) || !ot.integer(mat) || !ot.real(r[0])) {
            err = pot + ": bad record " + std::to_string(k + 1);
            return false;
        }
        a.itype[i] = (int)mat;
        a.h[i] = (float)r[0];
    }
    return true;
}

// Writes particles [first, first + n) with Fortran indices first+1.. (output.f).
inline bool write_set(const std::string& dir, const char* prefix, int dim, long long first,
                      long long n, const Arrays& a, std::string& err) {
    const std::string pre(prefix);
    const std::string paths[3] = {join(dir, (pre + "_xv.dat").c_str()),
                                  join(dir, (pre + "_state.dat").c_str()),
                                  join(dir, (pre + "_other.dat").c_str())};
    FILE* f[3] = {nullptr, nullptr, nullptr};
    for (int q = 0; q < 3; ++q)
        if (!(f[q] = std::fopen(paths[q].c_str(), "w"))) {
            err = "cannot create " + paths[q];
            for (int r = 0; r < q; ++r) std::fclose(f[r]);
            return false;
        }
    std::fprintf(f[0], "%12lld\n", n);  // list-directed write of the count
    std::string line;
    for (long long k = 0; k < n; ++k) {
        const long long i = first + k;
        const std::string idx = " " + fortran_i(i + 1, 6);
        line = idx;
        for (int d = 0; d < dim; ++d) line += "  " + fortran_e14_8(a.x[i * dim + d]);
        for (int d = 0; d < dim; ++d) line += "  " + fortran_e14_8(a.v[i * dim + d]);
        std::fprintf(f[0], "%s\n", line.c_str());
        line = idx;
        for (double q : {(double)a.mass[i], (double)a.rho[i], (double)a.p[i], (double)a.u[i]})
            line += "  " + fortran_e14_8(q);
        std::fprintf(f[1], "%s\n", line.c_str());
        line = idx + "  " + fortran_i(a.itype[i], 4) + "  " + fortran_e14_8(a.h[i]);
        std::fprintf(f[2], "%s\n", line.c_str());
    }
    bool ok = true;
    for (int q = 0; q < 3; ++q) ok = (std::fclose(f[q]) == 0) && ok;
    if (!ok) err = "write error in " + dir;
    return ok;
}

// Legacy VTK of armando.cu:1596-1670; 2D points get z = 0.
inline bool write_vtk(const std::string& path, int dim, long long n, const float* x, const float* v,
                      const float* rho, const float* p, const float* u, const int* itype,
                      std::string& err) {
    FILE* f = std::fopen(path.c_str(), "w");
    if (!f) {
        err = "cannot create " + path;
        return false;
    }
    std::fprintf(f, "# vtk DataFile Version 2.0\nUnstructured Grid Example\nASCII\n"
                    "DATASET UNSTRUCTURED_GRID\n");
    std::fprintf(f, "POINTS %lld float\n", n);
    for (long long i = 0; i < n; ++i)
        std::fprintf(f, "%+e %+e %+e \n", (double)x[i * dim], (double)x[i * dim + 1],
                     dim == 3 ? (double)x[i * dim + 2] : 0.0);
    std::fprintf(f, "CELLS %lld %lld \n", n, 2 * n);
    for (long long i = 0; i < n; ++i) std::fprintf(f, "%d %lld \n", 1, i);
    std::fprintf(f, "CELL_TYPES %lld \n", n);
    for (long long i = 0; i < n; ++i) std::fprintf(f, "%d \n", 1);
    std::fprintf(f, "POINT_DATA %lld \n", n);
    std::fprintf(f, "SCALARS material int 1 \nLOOKUP_TABLE default\n");
    for (long long i = 0; i < n; ++i) std::fprintf(f, "%+d \n", itype[i]);
    const float* fields[3] = {rho, p, u};
    const char* names[3] = {"density", "pressure", "energy"};
    for (int q = 0; q < 3; ++q) {
        std::fprintf(f, "SCALARS %s float 1 \nLOOKUP_TABLE default\n", names[q]);
        for (long long i = 0; i < n; ++i) std::fprintf(f, "%+e \n", (double)fields[q][i]);
    }
    std::fprintf(f, "VECTORS velocity float\n");
    for (long long i = 0; i < n; ++i)
        std::fprintf(f, "%+e %+e %+e \n", (double)v[i * dim], (double)v[i * dim + 1],
                     dim == 3 ? (double)v[i * dim + 2] : 0.0);
    if (std::fclose(f) != 0) {
        err = "write error in " + path;
        return false;
    }
    return true;
}

}  // namespace deck
}  // namespace ag
