"""The binary64 adjoints of the oracle against central differences
(h = 1e-3) of the binary64 forward, on CPU.  Relative error bound 1e-4 per
checked coordinate; a coordinate is checked only when no perturbation
changes a discrete choice (cube case, pixel, truncation, clamp).  The
dynamic-weight integrate, and marching cubes through edges whose two values
nearly agree, are curved enough that the plain quotient's truncation error
at h = 1e-3 reaches 1e-4 and more (it falls as h^2); those cases add one
Richardson step with h/2: (4 D(h/2) - D(h)) / 3.  Depth steps are h times
the truncation distance (the unit the normalised tsdf is measured in)."""
import numpy as np
import pytest

import oracle
from adjoint_util import Scene, smooth_volume

H = 1e-3
TOL = 1e-4


def test_mc_adjoint_central_differences():
    vol, cell = smooth_volume(24, seed=1)
    shape = vol.shape[:3]
    va, vb = oracle.mc_edges(vol)
    assert len(va) > 300
    rng = np.random.default_rng(0)
    G = rng.standard_normal((len(va), 3))
    g = oracle.mc_backward_f64(vol, cell, G).reshape(-1)

    def loss(F):
        return float((oracle.mc_positions_f64(F, va, vb, shape, cell) * G).sum())

    F0 = vol[..., 0].astype(np.float64).reshape(-1)
    cand = np.flatnonzero(np.abs(g) > 1e-3 * np.abs(g).max())
    rng.shuffle(cand)
    checked = 0
    for i in cand[:200]:
        if abs(F0[i]) <= 2 * H:
            continue
        # every incident edge well away from f_a == f_b keeps the difference quotient accurate
        incident = np.concatenate([vb[va == i], va[vb == i]])
        if np.min(np.abs(F0[incident] - F0[i])) < 0.25:
            continue
        vp = vol.copy()
        vp.reshape(-1, 2)[i, 0] += H
        vm = vol.copy()
        vm.reshape(-1, 2)[i, 0] -= H
        for v in (vp, vm):  # live topology unchanged
            ea, eb = oracle.mc_edges(v)
            assert np.array_equal(ea, va) and np.array_equal(eb, vb)
        Fp = F0.copy(); Fp[i] += H
        Fm = F0.copy(); Fm[i] -= H
        fd = (loss(Fp) - loss(Fm)) / (2 * H)
        assert abs(fd - g[i]) <= TOL * abs(g[i]), (i, fd, g[i])
        checked += 1
        if checked == 40:
            break
    assert checked >= 20


@pytest.mark.parametrize("dynamic", [False, True])
def test_integrate_adjoint_central_differences(dynamic):
    sc = Scene(n=24, frames=3, w=64, h=48, seed=2)
    F, W, sig0 = sc.integrate_f64(is_dynamic=dynamic)
    assert (W > 0).mean() > 0.01
    rng = np.random.default_rng(1)
    gF = np.where(W > 0, rng.standard_normal(sc.shape), 0.0)
    gW = np.where(W > 0, 0.1 * rng.standard_normal(sc.shape), 0.0)
    d64 = sc.depth.astype(np.float64)
    gd, gF0, gW0 = oracle.integrate_seq_backward_f64(sc.shape, sc.min_t, sc.max_t, sc.grid_s, sc.k_orc, sc.e_orc,
                                                     d64, gF, gW, is_dynamic=dynamic)
    assert np.count_nonzero(gd) > 50
    if not dynamic:
        # from the initial state (weight 0) the first observation replaces the tsdf outright
        assert np.all(gF0[W > 0] == 0.0)

    def loss(d):
        Fp, Wp, sig = sc.integrate_f64(depth=d, is_dynamic=dynamic)
        return float((gF * Fp).sum() + (gW * Wp).sum()), sig

    cand = np.flatnonzero(np.abs(gd.reshape(-1)) > 1e-3 * np.abs(gd).max())
    rng.shuffle(cand)
    checked = skipped = 0

    def quotient(j, h):
        dp = d64.copy().reshape(-1); dp[j] += h
        dm = d64.copy().reshape(-1); dm[j] -= h
        lp, sp = loss(dp.reshape(d64.shape))
        lm, sm = loss(dm.reshape(d64.shape))
        return (lp - lm) / (2 * h), sp == sig0 and sm == sig0

    hd = H * sc.min_t
    for j in cand[:120]:
        fd, ok = quotient(j, hd)
        if dynamic and ok:
            fd2, ok2 = quotient(j, hd / 2)
            fd, ok = (4 * fd2 - fd) / 3, ok2
        if not ok:
            skipped += 1
            continue
        an = gd.reshape(-1)[j]
        assert abs(fd - an) <= TOL * abs(an), (j, fd, an)
        checked += 1
        if checked == 30:
            break
    assert checked >= 15, (checked, skipped)


def test_integrate_adjoint_initial_volume():
    """dL/d(F0, W0) of a non-trivial starting volume against differences."""
    sc = Scene(n=20, frames=2, w=64, h=48, seed=3)
    vol0 = sc.integrate_f32()  # some fused state to start from
    F, W, sig0 = sc.integrate_f64(vol0=vol0)
    rng = np.random.default_rng(2)
    gF = np.where(W > 0, rng.standard_normal(sc.shape), 0.0)
    d64 = sc.depth.astype(np.float64)
    gd, gF0, gW0 = oracle.integrate_seq_backward_f64(sc.shape, sc.min_t, sc.max_t, sc.grid_s, sc.k_orc, sc.e_orc,
                                                     d64, gF, None, vol0=vol0)
    cand = np.flatnonzero((vol0[..., 1].reshape(-1) > 0) & (np.abs(gF0.reshape(-1)) > 0))
    assert len(cand) > 20
    checked = 0
    for i in cand[:20]:
        for ch, g in ((0, gF0), (1, gW0)):
            # binary64 forward of a float32 start: perturb through the binary64 route by scaling h
            vp = vol0.astype(np.float64).copy().reshape(-1, 2)
            hh = H * max(1.0, abs(vp[i, ch]))
            v32p = vol0.copy().reshape(-1, 2); v32p[i, ch] = np.float32(vp[i, ch] + hh)
            v32m = vol0.copy().reshape(-1, 2); v32m[i, ch] = np.float32(vp[i, ch] - hh)
            stepp = float(v32p[i, ch]) - vp[i, ch]
            stepm = vp[i, ch] - float(v32m[i, ch])
            Fp, Wp, sp = sc.integrate_f64(vol0=v32p.reshape(vol0.shape))
            Fm, Wm, sm = sc.integrate_f64(vol0=v32m.reshape(vol0.shape))
            assert sp == sig0 and sm == sig0
            fd = ((gF * Fp).sum() - (gF * Fm).sum()) / (stepp + stepm)
            an = g.reshape(-1)[i]
            assert abs(fd - an) <= 1e-3 * abs(an) + 1e-9, (i, ch, fd, an)
        checked += 1
    assert checked == 20


def test_chain_depth_to_positions_central_differences():
    """depth -> integrate -> marching cubes -> L = sum G . P."""
    sc = Scene(n=24, frames=3, w=64, h=48, seed=4)
    F, W, sig0 = sc.integrate_f64()
    vol = np.stack([F, W], axis=-1).astype(np.float32)
    va, vb = oracle.mc_edges(vol)
    assert len(va) > 100
    rng = np.random.default_rng(3)
    G = rng.standard_normal((len(va), 3))
    cell = sc.grid_s
    gF = oracle.mc_backward_f64(vol, cell, G)
    d64 = sc.depth.astype(np.float64)
    gd, _, _ = oracle.integrate_seq_backward_f64(sc.shape, sc.min_t, sc.max_t, sc.grid_s, sc.k_orc, sc.e_orc,
                                                 d64, gF, None)

    def loss(d):
        Fp, Wp, sig = sc.integrate_f64(depth=d)
        v = np.stack([Fp, Wp], axis=-1).astype(np.float32)
        ea, eb = oracle.mc_edges(v)
        same = np.array_equal(ea, va) and np.array_equal(eb, vb) and sig == sig0
        return float((oracle.mc_positions_f64(Fp, va, vb, sc.shape, cell) * G).sum()), same

    cand = np.flatnonzero(np.abs(gd.reshape(-1)) > 1e-2 * np.abs(gd).max())
    rng.shuffle(cand)

    def quotient(j, h):
        dp = d64.copy().reshape(-1); dp[j] += h
        dm = d64.copy().reshape(-1); dm[j] -= h
        lp, okp = loss(dp.reshape(d64.shape))
        lm, okm = loss(dm.reshape(d64.shape))
        return (lp - lm) / (2 * h), okp and okm

    # edges with f_b - f_a near 0 curve t strongly: one Richardson step
    hd = H * sc.min_t
    checked = 0
    for j in cand[:80]:
        f1, ok1 = quotient(j, hd)
        f2, ok2 = quotient(j, hd / 2)
        if not (ok1 and ok2):
            continue
        fd = (4 * f2 - f1) / 3
        an = gd.reshape(-1)[j]
        assert abs(fd - an) <= TOL * abs(an), (j, fd, an)
        checked += 1
        if checked == 20:
            break
    assert checked >= 10
