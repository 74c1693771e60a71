"""Rigid alignment of three-dimensional configurations, as the reference's
drivers apply it to the wells and to the frames of path.xyz
(instantonmod.f90:222-312 get_align / align_atoms, 346-376 rotate_atoms;
pimd_par.f90:159-183, rpi_ser.f90:74-92, instantonmod.f90:926-932).

A configuration is an array of natom * 3 numbers, x[atom*3 + dim]; atom
indices are 1-based as in the reference's namelists (atom1, atom2, atom3 =
1, 2, 3 by default, pimd_par.f90:84-86).  The same steps run in the C++
namelist drivers (host/align.hpp).  The reference stops for ndim != 3
(instantonmod.f90:234-237); supported() says whether a system can be aligned,
and the drivers leave other systems as read.
"""
import numpy as np

_TINY = 1.0e-10  # instantonmod.f90:283, 354


def supported(ndim, natom, atoms=(1, 2, 3)):
    return ndim == 3 and all(1 <= a <= natom for a in atoms)


def rotation(axis, theta):
    """The reference's matrix for a rotation about axis (1 = x, 2 = y, 3 = z):
    with (j, k) the other two axes in order, R[j,j] = R[k,k] = cos, R[j,k] =
    sin, R[k,j] = -sin (instantonmod.f90:355-370)."""
    j, k = [a for a in range(3) if a != axis - 1]
    r = np.eye(3)
    c, s = np.cos(theta), np.sin(theta)
    r[j, j] = r[k, k] = c
    r[j, k], r[k, j] = s, -s
    return r


def rotate_atoms(x, axis, theta):
    """x: (natom, 3); unchanged for |theta| <= 1e-10 (instantonmod.f90:354)."""
    if abs(theta) <= _TINY:
        return x
    return x @ rotation(axis, theta).T


def get_align(conf, atoms=(1, 2, 3)):
    """(theta1, theta2, theta3) of a configuration (instantonmod.f90:222-263)."""
    a1, a2, a3 = (a - 1 for a in atoms)
    x = np.asarray(conf, dtype=float).reshape(-1, 3)
    x = x - x[a1]
    w = x[a2] - x[a1]
    t1 = np.arctan2(w[1], w[0])
    x = rotate_atoms(x, 3, t1)
    w = x[a2] - x[a1]
    t2 = np.arctan2(w[2], w[0])
    x = rotate_atoms(x, 2, t2)
    w = x[a3] - x[a1]
    t3 = -np.arctan2(w[1], w[2])
    return float(t1), float(t2), float(t3)


def align_atoms(conf, angles, atoms=(1, 2, 3)):
    """conf moved by the given angles: its atom1 to the origin, then the z, y
    and x rotations; returned unchanged (not translated) when all three
    angles are below 1e-10 (instantonmod.f90:267-312)."""
    x = np.asarray(conf, dtype=float).reshape(-1, 3)
    t1, t2, t3 = angles
    if not any(abs(t) > _TINY for t in angles):
        return x.ravel().copy()
    x = x - x[atoms[0] - 1]
    x = rotate_atoms(x, 3, t1)
    x = rotate_atoms(x, 2, t2)
    x = rotate_atoms(x, 1, t3)
    return x.ravel()


def align_wells_ti(w1, w2, alignwell=False, atoms=(1, 2, 3)):
    """The wells as the TI driver leaves them (pimd_par.f90:159-165): well 1
    by its own angles, well 2 by its own angles with alignwell, else by well
    1's.  Returns (well1, well2, angles applied to well 2)."""
    t = get_align(w1, atoms)
    a1 = align_atoms(w1, t, atoms)
    if alignwell:
        t = get_align(w2, atoms)
    return a1, align_atoms(w2, t, atoms), t


def align_wells_rpi(w1, w2, atoms=(1, 2, 3)):
    """rpi_ser.f90:74-80 with alignwell: each well by its own angles."""
    return align_atoms(w1, get_align(w1, atoms), atoms), align_atoms(w2, get_align(w2, atoms), atoms)


def align_frames(frames, atoms=(1, 2, 3)):
    """The frames of path.xyz by the angles of the first
    (instantonmod.f90:926-932)."""
    if len(frames) == 0:
        return []
    t = get_align(frames[0], atoms)
    return [align_atoms(f, t, atoms) for f in frames]
