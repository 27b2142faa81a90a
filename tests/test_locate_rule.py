"""The fast voxel-location rule of the cell kernels (locate in
physicore_gb300/csrc/cells_device.cuh), restated with IEEE float32 numpy
arithmetic on the CPU: whenever the FP32 estimate decides (it lies farther than
its error bound from every integer), its voxel index and inside/outside verdict
must equal those of the reference's FP64 expression trunc((p - bbmin) / voxel)
with the bounds test !(q >= 0) || q >= n (mesh.cpp:37-61).  Positions are drawn
adversarially: every voxel boundary of several meshes, with offsets of 0..64 ulps
either side, plus uniform and out-of-range positions.
"""
import numpy as np

TOL_REL = np.float32(2.0 ** -21)
TOL_ABS = np.float32(2.0 ** -40)


def fast_rule(p, bbmin, voxel, n):
    """(decided, inside, idx) of the FP32 estimate, as the kernel evaluates it."""
    f32 = np.float32
    pf = p.astype(f32)
    mf = f32(bbmin)
    rf = f32(1.0 / voxel)
    qf = (pf - mf) * rf  # two float32 roundings, as __fsub_rn / __fmul_rn
    fl = np.floor(qf)
    tol = (np.abs(qf) + np.abs(pf) * rf) * TOL_REL + TOL_ABS
    with np.errstate(invalid="ignore"):
        decided = ((qf - fl) > tol) & ((fl + f32(1.0)) - qf > tol)
    inside = (fl >= 0) & (fl < f32(n))
    return decided, inside, fl.astype(np.float64)


def reference(p, bbmin, voxel, n):
    q = (p - float(bbmin)) / float(voxel)
    with np.errstate(invalid="ignore"):
        inside = (q >= 0.0) & (q < float(n))
    idx = np.where(inside, np.trunc(np.where(np.isfinite(q), q, 0.0)), -1.0)
    return inside, idx


def adversarial_positions(bbmin, voxel, n, rng):
    edges = bbmin + voxel * np.arange(-1, n + 2, dtype=np.float64)
    pts = [edges]
    x = edges.copy()
    lo = edges.copy()
    for _ in range(64):
        x = np.nextafter(x, np.inf)
        lo = np.nextafter(lo, -np.inf)
        pts += [x.copy(), lo.copy()]
    pts.append(rng.uniform(bbmin - voxel, bbmin + voxel * (n + 1), 200_000))
    pts.append(np.array([np.nan, np.inf, -np.inf, 1e30, -1e30, 0.0, -0.0]))
    return np.concatenate(pts)


def test_fast_rule_agrees_with_fp64_division():
    rng = np.random.default_rng(5)
    meshes = [(0, 20, 320), (0, 20, 200), (-100, 25, 37), (37, 7, 1000), (-2000, 10, 400), (5, 1, 4096),
              (0, 3, 1)]
    for bbmin, voxel, n in meshes:
        p = adversarial_positions(bbmin, voxel, n, rng)
        decided, inside, idx = fast_rule(p, bbmin, voxel, n)
        ref_inside, ref_idx = reference(p, bbmin, voxel, n)
        assert np.array_equal(inside[decided], ref_inside[decided]), (bbmin, voxel, n)
        both = decided & ref_inside
        assert np.array_equal(idx[both], ref_idx[both]), (bbmin, voxel, n)
        # the estimate decides almost everywhere away from boundaries
        uniform = slice(len(p) - 200_007, len(p) - 7)
        assert decided[uniform].mean() > 0.99, (bbmin, voxel, n, decided[uniform].mean())
        # and never on the NaN / infinite positions
        assert not decided[-7:-3].any()
