// Crossover temperature of a transition state (crossover.f90:49-71): the
// eigenvalues eta^2 of the mass-weighted Hessian H_ab / sqrt(m_a m_b), in
// ascending order, and beta_c = 2 pi / sqrt(-eta^2_min).  The reference fills
// the mass-weighted matrix with a second atom index that runs over 1..ndim
// (crossover.f90:56), which leaves the entries of atoms beyond ndim unset (and
// reads past the Hessian when natom < ndim); every atom pair is filled here.
#pragma once
#include <cmath>
#include <limits>
#include <vector>

#include "eigsym.hpp"

namespace pgh {

// hess: ndof x ndof (symmetric; dof = atom * ndim + dim); mass: natom.  eta2
// receives the ndof eigenvalues.  Returns beta_c, or NaN when no eigenvalue is
// negative (not a saddle point) or the eigensolver did not converge.
inline double crossover_beta(int ndim, int natom, const std::vector<double> &hess, const std::vector<double> &mass,
                             std::vector<double> &eta2) {
    const int nd = ndim * natom;
    std::vector<double> a((size_t)nd * nd), v;
    for (int i = 0; i < nd; i++)
        for (int j = 0; j < nd; j++)
            a[(size_t)i * nd + j] = hess[(size_t)i * nd + j] / std::sqrt(mass[i / ndim] * mass[j / ndim]);
    if (eigsym_jacobi(nd, a, eta2, v) < 0) return std::numeric_limits<double>::quiet_NaN();
    if (!(eta2[0] < 0.0)) return std::numeric_limits<double>::quiet_NaN();
    return 2.0 * 3.14159265358979 / std::sqrt(-eta2[0]);  // the reference's pi (instantonmod.f90:4)
}

}  // namespace pgh
