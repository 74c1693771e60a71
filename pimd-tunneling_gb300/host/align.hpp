// Rigid alignment of a three-dimensional configuration, as the reference's
// drivers apply it to the wells and to the frames of path.xyz
// (instantonmod.f90:222-312 get_align / align_atoms, 346-376 rotate_atoms;
// called at pimd_par.f90:159-165, rpi_par.f90:128-133, rpi_ser.f90:74-80 and
// instantonmod.f90:926-932):
//   origin at atom1; a rotation about z that brings atom2 - atom1 into the xz
//   plane (theta1); a rotation about y that brings it onto the x axis (theta2);
//   a rotation about x that brings atom3 - atom1 into the xz plane (theta3).
// Configurations are stored as x[atom*3 + dim]; atom indices are 1-based as
// in the reference's namelists (atom1 = 1, atom2 = 2, atom3 = 3 by default,
// pimd_par.f90:84-86).  The reference stops for ndim != 3
// (instantonmod.f90:234-237, 278-281) and reads out of bounds for natom < 3;
// the drivers here leave such configurations as they are (align_supported).
#pragma once
#include <cmath>
#include <vector>

namespace pgh {

struct AlignAngles {
    double theta1 = 0.0, theta2 = 0.0, theta3 = 0.0;
};

inline bool align_supported(int ndim, int natom, int atom1, int atom2, int atom3) {
    auto ok = [&](int a) { return a >= 1 && a <= natom; };
    return ndim == 3 && ok(atom1) && ok(atom2) && ok(atom3);
}

// Rotation of every atom about axis (1 = x, 2 = y, 3 = z) in the reference's
// sense: with (j, k) the other two axes in order, x_j' = cos t x_j + sin t x_k
// and x_k' = -sin t x_j + cos t x_k; nothing for |t| <= 1e-10
// (instantonmod.f90:346-376).
inline void rotate_atoms(std::vector<double> &x, int natom, int axis, double theta) {
    if (std::fabs(theta) <= 1.0e-10) return;
    const int j = axis == 1 ? 1 : 0, k = axis == 3 ? 1 : 2;
    const double c = std::cos(theta), s = std::sin(theta);
    for (int i = 0; i < natom; i++) {
        const double xj = x[(size_t)i * 3 + j], xk = x[(size_t)i * 3 + k];
        x[(size_t)i * 3 + j] = c * xj + s * xk;
        x[(size_t)i * 3 + k] = -s * xj + c * xk;
    }
}

// The three angles of a configuration (instantonmod.f90:222-263).
inline AlignAngles get_align(const std::vector<double> &xin, int natom, int atom1, int atom2, int atom3) {
    AlignAngles t;
    const int a1 = atom1 - 1, a2 = atom2 - 1, a3 = atom3 - 1;
    std::vector<double> x(xin.begin(), xin.begin() + (size_t)natom * 3);
    const double o[3] = {xin[(size_t)a1 * 3], xin[(size_t)a1 * 3 + 1], xin[(size_t)a1 * 3 + 2]};
    for (int i = 0; i < natom; i++)
        for (int d = 0; d < 3; d++) x[(size_t)i * 3 + d] -= o[d];
    auto rel = [&](int a, int d) { return x[(size_t)a * 3 + d] - x[(size_t)a1 * 3 + d]; };
    t.theta1 = std::atan2(rel(a2, 1), rel(a2, 0));
    rotate_atoms(x, natom, 3, t.theta1);
    t.theta2 = std::atan2(rel(a2, 2), rel(a2, 0));
    rotate_atoms(x, natom, 2, t.theta2);
    t.theta3 = -std::atan2(rel(a3, 1), rel(a3, 2));
    return t;
}

// A configuration moved by given angles (instantonmod.f90:267-312): atom1 of
// this configuration to the origin, then the z, y and x rotations.  With all
// three angles below 1e-10 the configuration is returned unchanged (not even
// translated), as in the reference.
inline std::vector<double> align_atoms(const std::vector<double> &xin, int natom, int atom1, const AlignAngles &t) {
    std::vector<double> x(xin.begin(), xin.begin() + (size_t)natom * 3);
    if (!(std::fabs(t.theta1) > 1.0e-10 || std::fabs(t.theta2) > 1.0e-10 || std::fabs(t.theta3) > 1.0e-10))
        return x;
    const int a1 = atom1 - 1;
    const double o[3] = {xin[(size_t)a1 * 3], xin[(size_t)a1 * 3 + 1], xin[(size_t)a1 * 3 + 2]};
    for (int i = 0; i < natom; i++)
        for (int d = 0; d < 3; d++) x[(size_t)i * 3 + d] -= o[d];
    rotate_atoms(x, natom, 3, t.theta1);
    rotate_atoms(x, natom, 2, t.theta2);
    rotate_atoms(x, natom, 1, t.theta3);
    return x;
}

// The wells as the TI driver leaves them (pimd_par.f90:159-165): well 1 by its
// own angles; well 2 by its own angles when own2 (namelist alignwell), else by
// well 1's.  Returns the angles applied to well 2.
inline AlignAngles align_wells_ti(std::vector<double> &w1, std::vector<double> &w2, int natom, int atom1, int atom2,
                                  int atom3, bool own2) {
    AlignAngles t = get_align(w1, natom, atom1, atom2, atom3);
    w1 = align_atoms(w1, natom, atom1, t);
    if (own2) t = get_align(w2, natom, atom1, atom2, atom3);
    w2 = align_atoms(w2, natom, atom1, t);
    return t;
}

// The frames of path.xyz by the angles of the first frame
// (instantonmod.f90:926-932).
inline void align_frames(std::vector<std::vector<double>> &frames, int natom, int atom1, int atom2, int atom3) {
    if (frames.empty()) return;
    const AlignAngles t = get_align(frames[0], natom, atom1, atom2, atom3);
    for (auto &f : frames) f = align_atoms(f, natom, atom1, t);
}

}  // namespace pgh
