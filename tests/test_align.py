"""Well and path alignment (instantonmod.f90:222-376 get_align / align_atoms /
rotate_atoms; pimd_par.f90:159-183, rpi_ser.f90:74-92,
instantonmod.f90:926-932), CPU only:

* a hand-worked configuration and the untranslated identity case;
* the Python restatement (python/align.py) against a loop-by-loop transcription
  of the reference's steps below, and the C++ header of the namelist drivers
  (host/align.hpp) against both;
* geometric invariants: atom1 at the origin, atom2 on the +x axis, atom3 in the
  xz plane, interatomic distances kept;
* the namelist drivers' --prepare-only output (aligned wells and path frames,
  aligned_wells.xyz / aligned_ends.xyz) for 3-D systems, and 2-D systems left
  as read."""
import json
import math
import os
import shutil
import subprocess

import numpy as np
import pytest

import align

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(ROOT, "pimd-tunneling_gb300", "lib")


# --- loop-by-loop transcription of the reference's three subroutines --------
def _rotate_loops(atoms, axis, theta):
    """instantonmod.f90:346-376: rotmatrix, then matmul per atom."""
    if abs(theta) <= 1e-10:
        return atoms
    j, k = {1: (2, 3), 2: (1, 3), 3: (1, 2)}[axis]
    R = [[0.0] * 3 for _ in range(3)]
    R[axis - 1][axis - 1] = 1.0
    R[j - 1][j - 1] = math.cos(theta)
    R[k - 1][k - 1] = math.cos(theta)
    R[k - 1][j - 1] = -math.sin(theta)
    R[j - 1][k - 1] = math.sin(theta)
    out = []
    for a in atoms:
        out.append([sum(R[r][c] * a[c] for c in range(3)) for r in range(3)])
    return out


def _get_align_loops(atomsin, a1, a2, a3):
    """instantonmod.f90:222-263."""
    origin = list(atomsin[a1 - 1])
    atoms = [[a[d] - origin[d] for d in range(3)] for a in atomsin]
    w = [atoms[a2 - 1][d] - atoms[a1 - 1][d] for d in range(3)]
    t1 = math.atan2(w[1], w[0])
    atoms = _rotate_loops(atoms, 3, t1)
    w = [atoms[a2 - 1][d] - atoms[a1 - 1][d] for d in range(3)]
    t2 = math.atan2(w[2], w[0])
    atoms = _rotate_loops(atoms, 2, t2)
    w = [atoms[a3 - 1][d] - atoms[a1 - 1][d] for d in range(3)]
    t3 = -math.atan2(w[1], w[2])
    return t1, t2, t3


def _align_atoms_loops(atomsin, t, a1):
    """instantonmod.f90:267-312."""
    if not any(abs(x) > 1e-10 for x in t):
        return [list(a) for a in atomsin]
    out = [[a[d] - atomsin[a1 - 1][d] for d in range(3)] for a in atomsin]
    out = _rotate_loops(out, 3, t[0])
    out = _rotate_loops(out, 2, t[1])
    out = _rotate_loops(out, 1, t[2])
    return out


def _rows(x):
    return [list(map(float, r)) for r in np.asarray(x, float).reshape(-1, 3)]


def _dists(x):
    x = np.asarray(x, float).reshape(-1, 3)
    return np.linalg.norm(x[:, None, :] - x[None, :, :], axis=-1)


# --- hand-worked cases ------------------------------------------------------
def test_known_answer():
    # atom2 - atom1 = (0, 1, 0): theta1 = pi/2 (onto +x), theta2 = 0;
    # atom3 - atom1 = (0, 1, 1) -> (1, 0, 1) after the z rotation: theta3 = 0
    w = np.array([1.0, 1.0, 1.0, 1.0, 2.0, 1.0, 1.0, 2.0, 2.0])
    t = align.get_align(w)
    assert t[0] == pytest.approx(math.pi / 2, abs=1e-15)
    assert abs(t[1]) < 1e-15 and abs(t[2]) < 1e-15  # round-off of cos(pi/2); below the 1e-10 skip
    np.testing.assert_allclose(align.align_atoms(w, t), [0, 0, 0, 1, 0, 0, 1, 0, 1], atol=1e-15)
    # atom3 - atom1 = (0, 1, 1) with atom2 already on x: theta3 = -pi/4 (y -> 0)
    w = np.array([0.0, 0.0, 0.0, 2.0, 0.0, 0.0, 0.0, 1.0, 1.0])
    t = align.get_align(w)
    assert t[0] == 0.0 and t[1] == 0.0
    assert t[2] == pytest.approx(-math.pi / 4, abs=1e-15)
    np.testing.assert_allclose(align.align_atoms(w, t), [0, 0, 0, 2, 0, 0, 0, 0, math.sqrt(2)], atol=1e-15)


def test_aligned_frame_is_not_translated():
    # all three angles 0: the reference copies the configuration as it is,
    # without moving atom1 to the origin (instantonmod.f90:283, 305)
    w = np.array([5.0, -1.0, 2.0, 7.0, -1.0, 2.0, 5.0, -1.0, 3.0])
    t = align.get_align(w)
    assert t == (0.0, 0.0, 0.0)
    np.testing.assert_array_equal(align.align_atoms(w, t), w)


# --- restatement vs transcription, invariants ------------------------------
CASES = [(3, (1, 2, 3)), (5, (1, 2, 3)), (9, (1, 2, 4)), (9, (1, 4, 7)), (18, (3, 1, 2))]


@pytest.mark.parametrize("natom,atoms", CASES)
def test_python_matches_transcription(natom, atoms):
    rng = np.random.default_rng(natom * 10 + atoms[1])
    for _ in range(20):
        w = rng.normal(size=natom * 3) * 2.0
        t = align.get_align(w, atoms)
        tl = _get_align_loops(_rows(w), *atoms)
        np.testing.assert_allclose(t, tl, rtol=0, atol=1e-14)
        x = align.align_atoms(w, t, atoms)
        np.testing.assert_allclose(x, np.ravel(_align_atoms_loops(_rows(w), tl, atoms[0])), rtol=0, atol=1e-13)
        xr = x.reshape(-1, 3)
        a1, a2, a3 = (a - 1 for a in atoms)
        np.testing.assert_allclose(xr[a1], 0.0, atol=1e-13)
        np.testing.assert_allclose(xr[a2, 1:], 0.0, atol=1e-12)
        assert xr[a2, 0] > 0.0
        assert abs(xr[a3, 1]) < 1e-12
        np.testing.assert_allclose(_dists(x), _dists(w), atol=1e-12)


def test_well_pairs_and_frames():
    rng = np.random.default_rng(7)
    w1 = rng.normal(size=27)
    w2 = w1 + 0.3 * rng.normal(size=27)
    # TI driver without alignwell: well 2 moved by well 1's angles about its own atom1
    a1, a2, t = align.align_wells_ti(w1, w2, alignwell=False)
    t1 = align.get_align(w1)
    assert t == t1
    np.testing.assert_allclose(a2, np.ravel(_align_atoms_loops(_rows(w2), t1, 1)), atol=1e-13)
    # with alignwell each well by its own angles; rpi_ser does the same
    b1, b2, t = align.align_wells_ti(w1, w2, alignwell=True)
    assert t == align.get_align(w2)
    c1, c2 = align.align_wells_rpi(w1, w2)
    np.testing.assert_array_equal(b1, c1)
    np.testing.assert_array_equal(b2, c2)
    np.testing.assert_array_equal(a1, b1)
    # path frames by the first frame's angles
    frames = [w1, 0.5 * (w1 + w2), w2]
    f = align.align_frames(frames)
    for fi, g in zip(f, frames):
        np.testing.assert_allclose(fi, np.ravel(_align_atoms_loops(_rows(g), t1, 1)), atol=1e-13)


def test_supported():
    assert align.supported(3, 3)
    assert not align.supported(2, 3)
    assert not align.supported(3, 1)
    assert not align.supported(3, 9, (1, 4, 10))


# --- the C++ header ---------------------------------------------------------
HARNESS = r'''
#include <cstdio>
#include <vector>
#include "align.hpp"
int main() {
    int natom, a1, a2, a3;
    if (std::scanf("%d %d %d %d", &natom, &a1, &a2, &a3) != 4) return 2;
    std::vector<double> x((size_t)natom * 3);
    for (auto &v : x)
        if (std::scanf("%lf", &v) != 1) return 2;
    const pgh::AlignAngles t = pgh::get_align(x, natom, a1, a2, a3);
    std::printf("%.17g %.17g %.17g\n", t.theta1, t.theta2, t.theta3);
    for (double v : pgh::align_atoms(x, natom, a1, t)) std::printf("%.17g\n", v);
    return 0;
}
'''


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    cxx = shutil.which(os.environ.get("CXX", "g++"))
    if not cxx:
        pytest.skip("no C++ compiler")
    d = tmp_path_factory.mktemp("align")
    src = d / "harness.cpp"
    src.write_text(HARNESS)
    exe = d / "harness"
    subprocess.run([cxx, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "pimd-tunneling_gb300", "host"), str(src),
                    "-o", str(exe)], check=True)
    return str(exe)


@pytest.mark.parametrize("natom,atoms", CASES)
def test_cpp_header_matches(harness, natom, atoms):
    rng = np.random.default_rng(100 + natom)
    for _ in range(5):
        w = rng.normal(size=natom * 3) * 3.0
        text = "%d %d %d %d\n" % ((natom,) + atoms) + "\n".join("%.17g" % v for v in w)
        out = np.array(subprocess.run([harness], input=text, capture_output=True, text=True,
                                      check=True).stdout.split(), dtype=float)
        np.testing.assert_allclose(out[:3], align.get_align(w, atoms), rtol=0, atol=1e-14)
        np.testing.assert_allclose(out[3:], align.align_atoms(w, align.get_align(w, atoms), atoms), rtol=0,
                                   atol=1e-13)


# --- the namelist drivers ---------------------------------------------------
def _write_inputs(d, w1, w2, frames, natom, ndim):
    (d / "masses.dat").write_text("".join("A%d 1837.0\n" % j for j in range(natom)))
    (d / "well1.dat").write_text("\n".join("%.17g" % v for v in w1) + "\n")
    (d / "well2.dat").write_text("\n".join("%.17g" % v for v in w2) + "\n")
    lines = []
    for i, f in enumerate(frames):
        lines += [" %d" % natom, " frame %d" % i]
        fr = np.asarray(f).reshape(natom, ndim)
        lines += [" A%d " % j + " ".join("%.17g" % v for v in fr[j]) for j in range(natom)]
    (d / "path.xyz").write_text("\n".join(lines) + "\n")


def _prepare(exe, text, cwd):
    path = os.path.join(LIB, exe)
    if not os.path.exists(path):
        pytest.skip("drivers not built")
    r = subprocess.run([path, "--prepare-only"], input=text, capture_output=True, text=True, cwd=cwd, timeout=60)
    assert r.returncode == 0, r.stderr
    return json.loads(r.stdout)


def _read_xyz(path, natom):
    toks = open(path).read().split("\n")
    frames, i = [], 0
    while i < len(toks) and toks[i].strip():
        rows = [list(map(float, toks[i + 2 + j].split()[1:])) for j in range(natom)]
        frames.append((toks[i + 1].strip(), np.array(rows).ravel() / 0.529177))
        i += 2 + natom
    return frames


@pytest.mark.parametrize("alignwell", [False, True])
def test_ti_driver_aligns(pg, tmp_path, alignwell):
    natom = 4
    rng = np.random.default_rng(3)
    w1 = rng.normal(size=natom * 3)
    w2 = w1 + 0.4 * rng.normal(size=natom * 3)
    frames = [w1, 0.5 * (w1 + w2) + 0.1, w2]
    _write_inputs(tmp_path, w1, w2, frames, natom, 3)
    text = ("&MCDATA n=8, ndim=3, natom=%d, readpath=.true., npath=3, alignwell=%s, atom3=4, pes='synth9' /"
            % (natom, ".true." if alignwell else ".false."))
    out = _prepare("pimd_ti", text, str(tmp_path))
    atoms = (1, 2, 4)
    e1, e2, t = align.align_wells_ti(w1, w2, alignwell=alignwell, atoms=atoms)
    np.testing.assert_allclose(out["well1"], e1, atol=1e-13)
    np.testing.assert_allclose(out["well2"], e2, atol=1e-13)
    np.testing.assert_allclose(np.array(out["path"]), np.array(align.align_frames(frames, atoms)), atol=1e-13)
    xyz = tmp_path / "aligned_wells.xyz"
    assert xyz.exists() == alignwell
    if alignwell:
        got = _read_xyz(str(xyz), natom)
        assert [c.split()[:2] for c, _ in got] == [["rotation", "angles:"]] * 2
        np.testing.assert_allclose(list(map(float, got[0][0].split()[2:])), t, atol=1e-15)
        np.testing.assert_allclose(got[0][1], e1, atol=1e-12)
        np.testing.assert_allclose(got[1][1], e2, atol=1e-12)


@pytest.mark.parametrize("alignwell", [False, True])
def test_rpi_driver_aligns(pg, tmp_path, alignwell):
    natom = 3
    rng = np.random.default_rng(4)
    w1 = rng.normal(size=9)
    w2 = w1 + 0.4 * rng.normal(size=9)
    frames = [w1, w2]
    _write_inputs(tmp_path, w1, w2, frames, natom, 3)
    text = ("&RPIDATA n=8, ndim=3, natom=3, readpath=.true., npath=2, alignwell=%s, pes='synth9' /"
            % (".true." if alignwell else ".false."))
    out = _prepare("rpi", text, str(tmp_path))
    e1, e2 = align.align_wells_rpi(w1, w2) if alignwell else (w1, w2)
    np.testing.assert_allclose(out["well1"], e1, atol=1e-13)
    np.testing.assert_allclose(out["well2"], e2, atol=1e-13)
    np.testing.assert_allclose(np.array(out["path"]), np.array(align.align_frames(frames)), atol=1e-13)
    xyz = tmp_path / "aligned_ends.xyz"
    assert xyz.exists() == alignwell
    if alignwell:
        got = _read_xyz(str(xyz), natom)
        assert [c for c, _ in got] == ["Well1", "Well2"]
        np.testing.assert_allclose(got[1][1], e2, atol=1e-12)


def test_two_dimensional_systems_are_left_as_read(pg, tmp_path):
    # the reference stops here (instantonmod.f90:234-237); the drivers keep the inputs
    rng = np.random.default_rng(5)
    w1, w2 = rng.normal(size=6), rng.normal(size=6)
    _write_inputs(tmp_path, w1, w2, [w1, w2], 3, 2)
    out = _prepare("pimd_ti", "&MCDATA n=8, ndim=2, natom=3, readpath=.true., npath=2, alignwell=.true., "
                              "pes='2dtest' /", str(tmp_path))
    np.testing.assert_array_equal(out["well1"], w1)
    np.testing.assert_array_equal(out["well2"], w2)
    assert not (tmp_path / "aligned_wells.xyz").exists()
