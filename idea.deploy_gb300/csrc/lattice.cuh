// Compile-time lattice and force-stencil tables for the sm_103a kernels.
//
// Vectors and their order are the reference's XIStencils / FStencils tables
// (idpy/LBM/LBM.py:74-185); the host checks that the caller's tables equal the
// compiled ones before any kernel runs.  Weights are not compiled in: the
// caller's doubles are passed at launch, so the force weights are exactly the
// values the reference prints (idpy/IdpyStencils/IdpyStencils.py:1538-1544).
#pragma once

#include <cstdint>

namespace sclbm {

#define SCLBM_HD __host__ __device__ __forceinline__

struct D2Q9 {
    static constexpr int D = 2, Q = 9;
    SCLBM_HD static constexpr int xi(int q, int d) {
        constexpr int t[9][2] = {{0, 0}, {1, 0}, {0, 1}, {-1, 0}, {0, -1},
                                 {1, 1}, {-1, 1}, {-1, -1}, {1, -1}};
        return t[q][d];
    }
};

struct D3Q19 {
    static constexpr int D = 3, Q = 19;
    SCLBM_HD static constexpr int xi(int q, int d) {
        constexpr int t[19][3] = {{0, 0, 0},
                                  {1, 0, 0}, {0, 1, 0}, {-1, 0, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1},
                                  {1, 1, 0}, {-1, 1, 0}, {-1, -1, 0}, {1, -1, 0},
                                  {1, 0, 1}, {-1, 0, 1}, {-1, 0, -1}, {1, 0, -1},
                                  {0, 1, 1}, {0, -1, 1}, {0, -1, -1}, {0, 1, -1}};
        return t[q][d];
    }
};

// ---- force stencils (isotropic, e2 = 1) -----------------------------------
struct D2E4 {
    static constexpr int D = 2, QE = 8, R = 1;
    SCLBM_HD static constexpr int e(int a, int d) {
        constexpr int t[8][2] = {{1, 0}, {0, 1}, {-1, 0}, {0, -1}, {1, 1}, {-1, 1}, {-1, -1}, {1, -1}};
        return t[a][d];
    }
};
struct D2E6 {
    static constexpr int D = 2, QE = 12, R = 2;
    SCLBM_HD static constexpr int e(int a, int d) {
        constexpr int t[12][2] = {{1, 0}, {0, 1}, {-1, 0}, {0, -1}, {1, 1}, {-1, 1}, {-1, -1}, {1, -1},
                                  {2, 0}, {0, 2}, {-2, 0}, {0, -2}};
        return t[a][d];
    }
};
struct D2E8 {
    static constexpr int D = 2, QE = 24, R = 2;
    SCLBM_HD static constexpr int e(int a, int d) {
        constexpr int t[24][2] = {{1, 0}, {0, 1}, {-1, 0}, {0, -1}, {1, 1}, {-1, 1}, {-1, -1}, {1, -1},
                                  {2, 0}, {0, 2}, {-2, 0}, {0, -2},
                                  {2, 1}, {1, 2}, {-1, 2}, {-2, 1}, {-2, -1}, {-1, -2}, {1, -2}, {2, -1},
                                  {2, 2}, {-2, 2}, {-2, -2}, {2, -2}};
        return t[a][d];
    }
};
struct D3E4 {
    static constexpr int D = 3, QE = 18, R = 1;
    SCLBM_HD static constexpr int e(int a, int d) {
        constexpr int t[18][3] = {{1, 0, 0}, {0, 1, 0}, {-1, 0, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1},
                                  {1, 1, 0}, {-1, 1, 0}, {-1, -1, 0}, {1, -1, 0},
                                  {0, 1, 1}, {0, -1, 1}, {0, -1, -1}, {0, 1, -1},
                                  {1, 0, 1}, {1, 0, -1}, {-1, 0, -1}, {-1, 0, 1}};
        return t[a][d];
    }
};
struct D3E6 {
    static constexpr int D = 3, QE = 32, R = 2;
    SCLBM_HD static constexpr int e(int a, int d) {
        constexpr int t[32][3] = {{1, 0, 0}, {0, 1, 0}, {-1, 0, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1},
                                  {1, 1, 0}, {-1, 1, 0}, {-1, -1, 0}, {1, -1, 0},
                                  {0, 1, 1}, {0, -1, 1}, {0, -1, -1}, {0, 1, -1},
                                  {1, 0, 1}, {1, 0, -1}, {-1, 0, -1}, {-1, 0, 1},
                                  {1, 1, 1}, {-1, 1, 1}, {-1, -1, 1}, {1, -1, 1},
                                  {1, 1, -1}, {-1, 1, -1}, {-1, -1, -1}, {1, -1, -1},
                                  {2, 0, 0}, {0, 2, 0}, {-2, 0, 0}, {0, -2, 0}, {0, 0, 2}, {0, 0, -2}};
        return t[a][d];
    }
};
struct D3E8 {
    static constexpr int D = 3, QE = 92, R = 2;
    SCLBM_HD static constexpr int e(int a, int d) {
        constexpr int t[92][3] = {
            {1, 0, 0}, {0, 1, 0}, {-1, 0, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1},
            {1, 1, 0}, {-1, 1, 0}, {-1, -1, 0}, {1, -1, 0},
            {0, 1, 1}, {0, -1, 1}, {0, -1, -1}, {0, 1, -1},
            {1, 0, 1}, {1, 0, -1}, {-1, 0, -1}, {-1, 0, 1},
            {1, 1, 1}, {-1, 1, 1}, {-1, -1, 1}, {1, -1, 1},
            {1, 1, -1}, {-1, 1, -1}, {-1, -1, -1}, {1, -1, -1},
            {2, 0, 0}, {0, 2, 0}, {-2, 0, 0}, {0, -2, 0}, {0, 0, 2}, {0, 0, -2},
            {2, 1, 0}, {2, -1, 0}, {2, 0, 1}, {2, 0, -1},
            {1, 2, 0}, {-1, 2, 0}, {0, 2, 1}, {0, 2, -1},
            {-2, 1, 0}, {-2, -1, 0}, {-2, 0, 1}, {-2, 0, -1},
            {1, -2, 0}, {-1, -2, 0}, {0, -2, 1}, {0, -2, -1},
            {1, 0, 2}, {-1, 0, 2}, {0, 1, 2}, {0, -1, 2},
            {1, 0, -2}, {-1, 0, -2}, {0, 1, -2}, {0, -1, -2},
            {2, 1, 1}, {2, -1, 1}, {2, -1, -1}, {2, 1, -1},
            {1, 2, 1}, {-1, 2, 1}, {-1, 2, -1}, {1, 2, -1},
            {-2, 1, 1}, {-2, -1, 1}, {-2, -1, -1}, {-2, 1, -1},
            {1, -2, 1}, {-1, -2, 1}, {-1, -2, -1}, {1, -2, -1},
            {1, 1, 2}, {-1, 1, 2}, {-1, -1, 2}, {1, -1, 2},
            {1, 1, -2}, {-1, 1, -2}, {-1, -1, -2}, {1, -1, -2},
            {2, 2, 0}, {-2, 2, 0}, {-2, -2, 0}, {2, -2, 0},
            {2, 0, 2}, {-2, 0, 2}, {-2, 0, -2}, {2, 0, -2},
            {0, 2, 2}, {0, -2, 2}, {0, -2, -2}, {0, 2, -2}};
        return t[a][d];
    }
};

// ---- monomials of the expanded collision -----------------------------------
// index layout (K = 1 + D + D(D+1)/2 + D + D*D):
//   0                  n          (dn = n - rho0 in shifted storage)
//   1 .. D             n u_a
//   next D(D+1)/2      n u_a u_b  (a <= b, row-major over the upper triangle)
//   next D             F_a
//   next D*D           F_a u_b    (a-major)
template <int D>
struct Mono {
    static constexpr int NU = 1;
    static constexpr int NUU = 1 + D;
    static constexpr int F = 1 + D + D * (D + 1) / 2;
    static constexpr int FU = F + D;
    static constexpr int K = FU + D * D;
    SCLBM_HD static constexpr int nuu(int a, int b) {  // a <= b
        return NUU + a * D - a * (a - 1) / 2 + (b - a);
    }
};

// Is the BGK coefficient of monomial k for population q nonzero?  Fixed by
// the lattice vector alone (w_q > 0, xi^2 - c2 != 0 for c2 = 1/3).
template <class L>
struct BgkNonzero {
    bool v[L::Q][Mono<L::D>::K];
    constexpr BgkNonzero() : v() {
        constexpr int D = L::D;
        using M = Mono<D>;
        for (int q = 0; q < L::Q; q++)
            for (int k = 0; k < M::K; k++) {
                bool nz = false;
                if (k == 0) nz = true;
                else if (k < M::NUU) nz = L::xi(q, k - M::NU) != 0;
                else if (k < M::F) {
                    for (int a = 0; a < D; a++)
                        for (int b = a; b < D; b++)
                            if (M::nuu(a, b) == k) nz = a == b ? true : (L::xi(q, a) * L::xi(q, b) != 0);
                } else if (k < M::FU) nz = L::xi(q, k - M::F) != 0;
                else {
                    const int a = (k - M::FU) / D, b = (k - M::FU) % D;
                    nz = a == b ? true : (L::xi(q, a) * L::xi(q, b) != 0);
                }
                v[q][k] = nz;
            }
    }
};
template <class L>
SCLBM_HD constexpr bool bgk_nonzero(int q, int k) {
    constexpr BgkNonzero<L> t{};
    return t.v[q][k];
}

}  // namespace sclbm
