// Host construction of the expanded collision operator (see coeffs.cpp).
#pragma once

#include <string>
#include <vector>

namespace sclbm {

struct CollisionSpec {
    int dim = 0, q = 0;
    const int *xi = nullptr;      // q*dim
    const double *w = nullptr;    // q
    double c2 = 0;
    int collision = 0;            // 0 BGK, 1 MRT
    double tau = 1;
    double omega = 0;             // BGK rate; > 0 overrides 1/tau
    const double *mrt_s = nullptr;  // q*q relaxation matrix (moment basis)
    int literals = 0;             // 0 round to 15 digits, 1 exact
};

struct CollisionTables {
    int K = 0;
    bool a_diag = true;
    std::vector<double> A;    // q*q population operator
    std::vector<double> B;    // q*K monomial coefficients
    std::vector<double> Beq;  // q*K equilibrium coefficients (initialisation)
};

int build_collision(const CollisionSpec &s, CollisionTables &t, std::string &err);

// noise operator of the fluctuating (Gross 2011) step: m2var[j] = -2 var_j and
// coef[q*NR + j], the weight of random moment j in noise population q (NR = q-dim-1)
int build_noise(const CollisionSpec &s, double kBT, double n0, std::vector<double> &m2var,
                std::vector<double> &coef, std::string &err);

}  // namespace sclbm
