// Host-side construction of the collision operator, in exact rational arithmetic.
//
// The reference generates each post-collision population as an expanded sympy
// expression and prints its coefficients with evalf() (15 significant digits):
//   BGK + Guo   idpy/LBM/Collisions.py:163-185,251-273, idpy/LBM/Forcings.py:104-127
//   MRT + Guo   idpy/LBM/Collisions.py:96-160,275-316,  idpy/LBM/Forcings.py:129-181
//   equilibria  idpy/LBM/Equilibria.py:107-210
//   bases       idpy/IdpyStencils/IdpyStencils.py:838-1043 (invertible Hermite set,
//               Gram-Schmidt W-orthogonalised set)
// Here the same operator is assembled from exact rationals (the double inputs
// omega, S are taken at their exact binary values) and each coefficient is
// rounded once: to the 15-digit literal the reference prints
// (SCLBM_LIT_ROUND15) or to the nearest double (SCLBM_LIT_EXACT).  The result
// is a table per population q over the monomials of lattice.cuh:
//     f*_q = sum_j A[q][j] f_j + sum_k B[q][k] m_k
// which the kernels evaluate (BGK: A diagonal).
#include "coeffs.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

namespace sclbm {

using i128 = __int128;
using u128 = unsigned __int128;

namespace {

u128 ugcd(u128 a, u128 b) {
    while (b) {
        u128 t = a % b;
        a = b;
        b = t;
    }
    return a;
}

struct Rat {
    i128 n = 0, d = 1;
    Rat() = default;
    Rat(long long v) : n(v), d(1) {}
    static Rat make(i128 n, i128 d) {
        if (d == 0) throw std::domain_error("zero denominator");
        if (d < 0) { n = -n; d = -d; }
        u128 g = ugcd(n < 0 ? (u128)(-n) : (u128)n, (u128)d);
        Rat r;
        if (g > 1) { n /= (i128)g; d /= (i128)g; }
        r.n = n;
        r.d = d;
        return r;
    }
    bool zero() const { return n == 0; }
};

i128 mul_chk(i128 a, i128 b) {
    i128 r;
    if (__builtin_mul_overflow(a, b, &r)) throw std::overflow_error("rational overflow");
    return r;
}
i128 add_chk(i128 a, i128 b) {
    i128 r;
    if (__builtin_add_overflow(a, b, &r)) throw std::overflow_error("rational overflow");
    return r;
}

Rat operator*(const Rat &a, const Rat &b) {
    if (a.zero() || b.zero()) return Rat(0);
    // cross-reduce first to keep numbers small
    u128 g1 = ugcd(a.n < 0 ? (u128)(-a.n) : (u128)a.n, (u128)b.d);
    u128 g2 = ugcd(b.n < 0 ? (u128)(-b.n) : (u128)b.n, (u128)a.d);
    return Rat::make(mul_chk(a.n / (i128)g1, b.n / (i128)g2), mul_chk(a.d / (i128)g2, b.d / (i128)g1));
}
Rat operator+(const Rat &a, const Rat &b) {
    if (a.zero()) return b;
    if (b.zero()) return a;
    u128 g = ugcd((u128)a.d, (u128)b.d);
    i128 da = a.d / (i128)g, db = b.d / (i128)g;
    return Rat::make(add_chk(mul_chk(a.n, db), mul_chk(b.n, da)), mul_chk(a.d, db));
}
Rat operator-(const Rat &a) { Rat r = a; r.n = -r.n; return r; }
Rat operator-(const Rat &a, const Rat &b) { return a + (-b); }
Rat operator/(const Rat &a, const Rat &b) {
    if (b.zero()) throw std::domain_error("division by zero");
    Rat inv = Rat::make(b.d, b.n);
    return a * inv;
}

// exact value of a double
Rat from_double(double x) {
    if (!std::isfinite(x)) throw std::domain_error("non-finite input");
    if (x == 0) return Rat(0);
    int e;
    double m = std::frexp(x, &e);  // x = m 2^e, 0.5 <= |m| < 1
    long long mi = (long long)std::ldexp(m, 53);
    e -= 53;
    if (e >= 0) {
        if (e > 70) throw std::overflow_error("exponent");
        return Rat::make((i128)mi << e, 1);
    }
    if (-e > 120) throw std::overflow_error("exponent");
    return Rat::make(mi, (i128)1 << (-e));
}

// exact decimal expansion of |r| with `sig` significant digits, rounded half-even;
// returns mantissa digits and the decimal exponent of the first digit
std::string to_sci(const Rat &r, int sig) {
    if (r.zero()) return "0";
    bool neg = r.n < 0;
    u128 num = neg ? (u128)(-r.n) : (u128)r.n, den = (u128)r.d;
    // integer part and its digits
    u128 ip = num / den, rem = num % den;
    std::string digits;
    int exp10 = -1;
    if (ip > 0) {
        std::string s;
        u128 t = ip;
        while (t) { s.push_back(char('0' + (int)(t % 10))); t /= 10; }
        for (auto it = s.rbegin(); it != s.rend(); ++it) digits.push_back(*it);
        exp10 = (int)digits.size() - 1;
    }
    // fractional digits
    bool started = ip > 0;
    int frac_pos = 0;
    while ((int)digits.size() < sig + 2) {
        if (rem > ((u128)-1) / 10) throw std::overflow_error("decimal expansion");
        rem *= 10;
        int dgt = (int)(rem / den);
        rem %= den;
        frac_pos++;
        if (!started) {
            if (dgt == 0) {
                if (frac_pos > 400) return "0";
                continue;
            }
            started = true;
            exp10 = -frac_pos;
        }
        digits.push_back(char('0' + dgt));
    }
    bool sticky = rem != 0;
    // round digits[0..sig) half-even using digits[sig], digits[sig+1], sticky
    std::string keep = digits.substr(0, sig);
    int next = digits[sig] - '0';
    bool more = sticky;
    for (size_t i = sig + 1; i < digits.size(); i++) more = more || digits[i] != '0';
    bool up = next > 5 || (next == 5 && (more || ((keep.back() - '0') & 1)));
    if (up) {
        int i = sig - 1;
        while (i >= 0 && keep[i] == '9') { keep[i] = '0'; i--; }
        if (i < 0) { keep.insert(keep.begin(), '1'); keep.pop_back(); exp10++; }
        else keep[i]++;
    }
    char buf[64];
    std::snprintf(buf, sizeof(buf), "e%d", exp10);
    std::string out = std::string(neg ? "-" : "") + keep[0] + "." + keep.substr(1) + buf;
    return out;
}

double round_sig(const Rat &r, int sig) {
    if (r.zero()) return 0.0;
    std::string s = to_sci(r, sig);
    return std::strtod(s.c_str(), nullptr);
}

double to_double(const Rat &r) { return round_sig(r, 40); }

// small rational equal to a double (4/9, 1/3, ...), else its exact value
Rat recognize(double x) {
    Rat exact = from_double(x);
    // continued fraction convergents
    double v = x;
    long long h0 = 0, h1 = 1, k0 = 1, k1 = 0;
    for (int it = 0; it < 40; it++) {
        double a = std::floor(v);
        if (std::fabs(a) > 1e12) break;
        long long ai = (long long)a;
        long long h2 = ai * h1 + h0, k2 = ai * k1 + k0;
        if (k2 > 1000000 || k2 <= 0) break;
        h0 = h1; h1 = h2; k0 = k1; k1 = k2;
        if ((double)h1 / (double)k1 == x) return Rat::make(h1, k1);
        double f = v - a;
        if (f == 0) break;
        v = 1.0 / f;
    }
    return exact;
}

using Mat = std::vector<std::vector<Rat>>;

Mat matmul(const Mat &A, const Mat &B) {
    size_t n = A.size(), m = B[0].size(), p = B.size();
    Mat C(n, std::vector<Rat>(m));
    for (size_t i = 0; i < n; i++)
        for (size_t k = 0; k < p; k++) {
            if (A[i][k].zero()) continue;
            for (size_t j = 0; j < m; j++)
                if (!B[k][j].zero()) C[i][j] = C[i][j] + A[i][k] * B[k][j];
        }
    return C;
}

Mat inverse(Mat a) {
    size_t n = a.size();
    for (size_t i = 0; i < n; i++) {
        a[i].resize(2 * n);
        for (size_t j = 0; j < n; j++) a[i][n + j] = Rat(i == j ? 1 : 0);
    }
    for (size_t c = 0; c < n; c++) {
        size_t p = c;
        while (p < n && a[p][c].zero()) p++;
        if (p == n) throw std::domain_error("singular moment basis");
        std::swap(a[c], a[p]);
        Rat pv = a[c][c];
        for (auto &x : a[c]) x = x / pv;
        for (size_t i = 0; i < n; i++) {
            if (i == c || a[i][c].zero()) continue;
            Rat f = a[i][c];
            for (size_t j = 0; j < 2 * n; j++)
                if (!a[c][j].zero()) a[i][j] = a[i][j] - f * a[c][j];
        }
    }
    Mat inv(n, std::vector<Rat>(n));
    for (size_t i = 0; i < n; i++)
        for (size_t j = 0; j < n; j++) inv[i][j] = a[i][n + j];
    return inv;
}

bool independent(const Mat &basis, const std::vector<Rat> &r) {
    Mat m = basis;
    m.push_back(r);
    size_t rows = m.size(), cols = r.size(), rank = 0;
    for (size_t c = 0; c < cols && rank < rows; c++) {
        size_t p = rank;
        while (p < rows && m[p][c].zero()) p++;
        if (p == rows) continue;
        std::swap(m[rank], m[p]);
        for (size_t i = 0; i < rows; i++) {
            if (i == rank || m[i][c].zero()) continue;
            Rat f = m[i][c] / m[rank][c];
            for (size_t j = c; j < cols; j++)
                if (!m[rank][j].zero()) m[i][j] = m[i][j] - f * m[rank][j];
        }
        rank++;
    }
    return rank == rows;
}

// c_s^n H^(n)_{idx}(xi / c_s): H_{i+a} = x_a H_i - c2 sum_{k: i_k = a} H_{i \ k}
Rat hermite(const std::vector<int> &idx, const int *x, const Rat &c2) {
    if (idx.empty()) return Rat(1);
    int a = idx.back();
    std::vector<int> rest(idx.begin(), idx.end() - 1);
    Rat v = Rat(x[a]) * hermite(rest, x, c2);
    for (size_t k = 0; k < rest.size(); k++) {
        if (rest[k] != a) continue;
        std::vector<int> r2 = rest;
        r2.erase(r2.begin() + k);
        v = v - c2 * hermite(r2, x, c2);
    }
    return v;
}

void tuples_rec(int D, int order, int start, std::vector<int> &cur, std::vector<std::vector<int>> &out) {
    if ((int)cur.size() == order) { out.push_back(cur); return; }
    for (int a = start; a < D; a++) {
        cur.push_back(a);
        tuples_rec(D, order, a, cur, out);
        cur.pop_back();
    }
}

// (Mn, Mw): invertible Hermite set and its W-orthogonal Gram-Schmidt form
void hermite_bases(int D, int Q, const int *xi, const std::vector<Rat> &W, const Rat &c2,
                   Mat &Mn, Mat &Mw) {
    const int search_depth = 6;
    Mat rows;
    rows.push_back(std::vector<Rat>(Q, Rat(1)));
    int count = 1, order = 1;
    while (count < Q + search_depth) {
        std::vector<std::vector<int>> tups;
        std::vector<int> cur;
        tuples_rec(D, order, 0, cur, tups);
        for (auto &t : tups) {
            std::vector<Rat> r(Q);
            bool nz = false;
            for (int i = 0; i < Q; i++) {
                r[i] = hermite(t, xi + i * D, c2);
                nz = nz || !r[i].zero();
            }
            if (nz) { rows.push_back(r); count++; }
        }
        order++;
        if (order > 12) break;
    }
    Mn.clear();
    for (auto &r : rows) {
        if ((int)Mn.size() == Q) break;
        if (independent(Mn, r)) Mn.push_back(r);
    }
    if ((int)Mn.size() != Q) throw std::domain_error("no invertible Hermite set");
    auto prod = [&](const std::vector<Rat> &a, const std::vector<Rat> &b) {
        Rat s(0);
        for (int i = 0; i < Q; i++) s = s + a[i] * b[i] * W[i];
        return s;
    };
    Mw.clear();
    Mw.push_back(Mn[0]);
    for (int i = 1; i < Q; i++) {
        std::vector<Rat> v = Mn[i];
        for (auto &u : Mw) {
            Rat p = prod(Mn[i], u) / prod(u, u);
            if (p.zero()) continue;
            for (int j = 0; j < Q; j++) v[j] = v[j] - p * u[j];
        }
        Mw.push_back(v);
    }
}

// monomial coefficients of omega*feq_q + g*Fguo_q (g = forcing prefactor) for
// one population, layout of lattice.cuh
void bgk_monomials(int D, const int *x, const Rat &wq, const Rat &c2, const Rat &om, const Rat &g,
                   std::vector<Rat> &out) {
    const int NU = 1, NUU = 1 + D, F = 1 + D + D * (D + 1) / 2, FU = F + D;
    const int K = FU + D * D;
    out.assign(K, Rat(0));
    Rat c4 = c2 * c2;
    out[0] = om * wq;
    for (int a = 0; a < D; a++) out[NU + a] = om * wq * Rat(x[a]) / c2;
    int k = NUU;
    for (int a = 0; a < D; a++)
        for (int b = a; b < D; b++, k++) {
            if (a == b) out[k] = om * wq * (Rat(x[a] * x[a]) - c2) / (Rat(2) * c4);
            else out[k] = om * wq * Rat(x[a] * x[b]) / c4;
        }
    for (int a = 0; a < D; a++) out[F + a] = g * wq * Rat(x[a]) / c2;
    for (int a = 0; a < D; a++)
        for (int b = 0; b < D; b++)
            out[FU + a * D + b] = g * wq * (Rat(x[a] * x[b]) - (a == b ? c2 : Rat(0))) / c4;
}

}  // namespace

int build_collision(const CollisionSpec &s, CollisionTables &t, std::string &err) {
    try {
        const int D = s.dim, Q = s.q;
        const int K = 1 + D + D * (D + 1) / 2 + D + D * D;
        std::vector<Rat> W(Q);
        for (int i = 0; i < Q; i++) W[i] = recognize(s.w[i]);
        Rat c2 = recognize(s.c2);
        auto lit = [&](const Rat &r) {
            return s.literals == 0 ? round_sig(r, 15) : to_double(r);
        };
        t.K = K;
        t.A.assign((size_t)Q * Q, 0.0);
        t.B.assign((size_t)Q * K, 0.0);
        t.Beq.assign((size_t)Q * K, 0.0);
        t.a_diag = (s.collision == 0);
        // equilibrium (init): omega = 1, no forcing
        for (int q = 0; q < Q; q++) {
            std::vector<Rat> m;
            bgk_monomials(D, s.xi + q * D, W[q], c2, Rat(1), Rat(0), m);
            for (int k = 0; k < K; k++) t.Beq[(size_t)q * K + k] = lit(m[k]);
        }
        if (s.collision == 0) {
            Rat om = from_double(s.omega > 0 ? s.omega : 1.0 / s.tau);
            Rat g = Rat(1) - om / Rat(2);
            for (int q = 0; q < Q; q++) {
                std::vector<Rat> m;
                bgk_monomials(D, s.xi + q * D, W[q], c2, om, g, m);
                for (int k = 0; k < K; k++) t.B[(size_t)q * K + k] = lit(m[k]);
                t.A[(size_t)q * Q + q] = lit(Rat(1) - om);
            }
        } else {
            Mat Mn, Mw;
            hermite_bases(D, Q, s.xi, W, c2, Mn, Mw);
            Mat Mwi = inverse(Mw), Mni = inverse(Mn);
            Mat S(Q, std::vector<Rat>(Q)), IS(Q, std::vector<Rat>(Q)), IH(Q, std::vector<Rat>(Q));
            for (int i = 0; i < Q; i++)
                for (int j = 0; j < Q; j++) {
                    S[i][j] = from_double(s.mrt_s[(size_t)i * Q + j]);
                    IS[i][j] = Rat(i == j ? 1 : 0) - S[i][j];
                    IH[i][j] = Rat(i == j ? 1 : 0) - S[i][j] / Rat(2);
                }
            Mat A = matmul(Mwi, matmul(IS, Mw));
            Mat Beq = matmul(Mwi, matmul(S, Mw));
            Mat C = matmul(Mni, matmul(IH, Mn));
            std::vector<std::vector<Rat>> feq(Q), fg(Q);
            for (int j = 0; j < Q; j++) {
                bgk_monomials(D, s.xi + j * D, W[j], c2, Rat(1), Rat(0), feq[j]);
                bgk_monomials(D, s.xi + j * D, W[j], c2, Rat(0), Rat(1), fg[j]);
            }
            const int F = 1 + D + D * (D + 1) / 2;
            for (int i = 0; i < Q; i++) {
                std::vector<Rat> acc(K);
                for (int j = 0; j < Q; j++) {
                    for (int k = 0; k < F; k++)
                        if (!Beq[i][j].zero() && !feq[j][k].zero()) acc[k] = acc[k] + Beq[i][j] * feq[j][k];
                    for (int k = F; k < K; k++)
                        if (!C[i][j].zero() && !fg[j][k].zero()) acc[k] = acc[k] + C[i][j] * fg[j][k];
                    t.A[(size_t)i * Q + j] = lit(A[i][j]);
                }
                for (int k = 0; k < K; k++) t.B[(size_t)i * K + k] = lit(acc[k]);
            }
        }
        return 0;
    } catch (const std::exception &e) {
        err = e.what();
        return 1;
    }
}

// Noise operator of the fluctuating step (Gross et al. 2011; GrossShanChenMultiPhase,
// idpy/LBM/Fluctuations.py:40-165): the random moments are the W-orthogonal Hermite
// moments k = D+1 .. Q-1, so the noise populations are
//     rpop_q = sum_k Mw^-1[q][k] Rm_{k-D-1}                       (Fluctuations.py:158-163)
// and moment k has the variance (GetVariances, Fluctuations.py:72-97)
//     var_k = norm_k kBT (2 - 1/tau) / tau / c_s^2 n0,  norm_k = sum_q w_q Mw[k][q]^2.
// var_k is evaluated as the reference does: each product and quotient rounded to
// double (sympy Floats of 53 bits), tau = 1/(1/tau) (the kernel gets tau as
// 1/OMEGA).  SCLBM_LIT_ROUND15 then prints var_k and each coefficient with 15
// significant digits; SCLBM_LIT_EXACT keeps var_k and rounds the exact
// coefficients once to double.
int build_noise(const CollisionSpec &s, double kBT, double n0, std::vector<double> &m2var,
                std::vector<double> &coef, std::string &err) {
    try {
        const int D = s.dim, Q = s.q, NR = Q - D - 1;
        if (NR <= 0) throw std::domain_error("no random moments");
        std::vector<Rat> W(Q);
        for (int i = 0; i < Q; i++) W[i] = recognize(s.w[i]);
        const Rat c2 = recognize(s.c2);
        Mat Mn, Mw;
        hermite_bases(D, Q, s.xi, W, c2, Mn, Mw);
        const Mat Mwi = inverse(Mw);
        m2var.assign(NR, 0.0);
        coef.assign((size_t)Q * NR, 0.0);
        const double tau = 1.0 / (1.0 / s.tau);
        for (int j = 0; j < NR; j++) {
            const int k = D + 1 + j;
            Rat norm(0);
            for (int q = 0; q < Q; q++) norm = norm + W[q] * Mw[k][q] * Mw[k][q];
            double var = to_double(norm) * kBT;
            var = var * (2.0 - 1.0 / tau);
            var = var / tau;
            var = var / s.c2;
            var = var * n0;
            if (s.literals == 0 && var != 0.0) {
                char buf[40];
                std::snprintf(buf, sizeof buf, "%.14e", var);
                var = std::strtod(buf, nullptr);
            }
            m2var[j] = -2.0 * var;
            for (int q = 0; q < Q; q++)
                coef[(size_t)q * NR + j] = s.literals == 0 ? round_sig(Mwi[q][k], 15) : to_double(Mwi[q][k]);
        }
        return 0;
    } catch (const std::exception &e) {
        err = e.what();
        return 1;
    }
}

}  // namespace sclbm
