"""Per-pixel z-test of a GPU image against the CPU oracle, with its null
distribution measured on the oracle itself (helper of the GPU parity tests).

For every pixel and colour channel, a test image's mean over S samples is
compared with a reference mean over N samples of the oracle (N = 16 S, on
streams disjoint from the test image's):

    z = (m_test - m_ref) / sqrt(v (1/S + 1/N)),

v the pooled per-sample variance of both sample sets, so the oracle's own
Monte Carlo noise is in the test. A pixel-channel exceeds at |z| > 4.

Null distribution. At tens of samples per pixel the means of these
estimators are far from Gaussian: a pixel's radiance is a rare bright sample
(the sun through glass, a caustic, a light reached by a BSDF sample) on top
of a dim majority, so even the reference exceeds 4 sigma on far more than
the Gaussian 6.3e-5 of its pixels. The same statistic is therefore computed
for null images: S further oracle samples per pixel on other sets of
streams, against the same reference; three such null images give the
spread of the null counts. Exceedances are counted per pixel (any channel),
since a path's three channels move together. The GPU image passes when its
count is within the 99.9% Poisson bound of an expectation equal to the
largest null count (or the Gaussian expectation, when larger); the same
holds on 8x8-pixel blocks, and the mean z (bias) must match the nulls' to 4
standard errors. Counts are printed for all images.
"""
from __future__ import annotations

import math

import numpy as np

P_EXCEED_4SIGMA = 6.334248366623996e-05   # 2 (1 - Phi(4))


def poisson_bound(expected: float, q: float = 0.999) -> int:
    """Smallest k with P(X <= k) >= q for X ~ Poisson(expected): terms summed
    in log space (exp(-expected) underflows for large expectations), the
    normal approximation beyond 1000."""
    lam = float(expected)
    if lam > 1000.0:
        return int(np.ceil(lam + 3.0902 * np.sqrt(lam) + 1.0))
    cdf, k = 0.0, 0
    while True:
        cdf += math.exp(-lam + k * math.log(lam) - math.lgamma(k + 1)) if lam > 0 else (1.0 if k == 0 else 0.0)
        if cdf >= q or k > 10 * lam + 100:
            return k
        k += 1


def _z(ts, ts2, S, cs, cs2, N):
    mt, mc = ts / S, cs / N
    vt = np.maximum(ts2 / S - mt * mt, 0.0) * S / max(S - 1, 1)
    vc = np.maximum(cs2 / N - mc * mc, 0.0) * N / max(N - 1, 1)
    d = mt - mc
    v = ((S - 1) * vt + (N - 1) * vc + S * N / (S + N) * d * d) / (S + N - 1)
    var_mean = v * (1.0 / S + 1.0 / N)
    tiny = np.abs(d) <= 1e-6 * (1.0 + np.abs(mc))          # equal to float resolution (e.g. pure background)
    se = np.sqrt(var_mean)
    z = np.where(tiny, 0.0, d / np.where(se > 0, se, np.inf))
    z = np.where(~tiny & (se == 0), np.inf, z)
    return z, d, var_mean, mc


def _blocks(a, block):
    h, w = a.shape[:2]
    hb, wb = h // block, w // block
    return a[:hb * block, :wb * block].reshape(hb, block, wb, block, -1).sum((1, 3))


def _counts(z, d, var_mean, mc, block):
    """Exceedances of pixels (any channel beyond 4 sigma: the three channels
    of a path are strongly correlated), of 8x8 blocks likewise, and the mean z."""
    zmax = np.abs(z).max(-1)
    zf = z[np.isfinite(z)]
    out = {"n": zmax.size, "exceed": int((zmax > 4.0).sum()), "mean_z": float(zf.mean()),
           "sem_z": float(zf.std() / np.sqrt(zf.size))}
    if z.shape[0] >= block and z.shape[1] >= block:
        bd, bv = _blocks(d, block), _blocks(var_mean, block)
        zb = bd / np.sqrt(np.maximum(bv, 1e-300))
        zb = np.where(np.abs(bd) <= 1e-6 * (1.0 + np.abs(_blocks(mc, block))), 0.0, zb)
        zbm = np.abs(zb).max(-1)
        out.update(blocks=zbm.size, block_exceed=int((zbm > 4.0).sum()), block_max=float(zbm.max()))
    return out


def allowed(null_counts, n: int) -> int:
    """Exceedances allowed: the 99.9% Poisson bound of an expected count
    equal to the largest count among the null images (or the Gaussian
    expectation, three channels per pixel, when larger)."""
    return poisson_bound(max(float(max(null_counts)), 3.0 * n * P_EXCEED_4SIGMA))


def ztest(name, ts, ts2, S, cs, cs2, N, nulls, block=8):
    """ts/ts2: the test image's per-pixel sums and sums of squares of S
    samples; cs/cs2: the oracle reference's, N samples; nulls: a list of
    (sums, sums of squares) of oracle null images of S samples each (all
    streams disjoint)."""
    z, d, vm, mc = _z(ts, ts2, S, cs, cs2, N)
    g = _counts(z, d, vm, mc, block)
    os_ = []
    for ns, ns2 in nulls:
        z0, d0, vm0, _ = _z(ns, ns2, S, cs, cs2, N)
        os_.append(_counts(z0, d0, vm0, mc, block))
    zmax = np.abs(z).max(-1)
    worst = np.argsort(-zmax.ravel())[:4]
    idx = [tuple(int(i) for i in np.unravel_index(k, zmax.shape)) for k in worst]
    lim = allowed([o["exceed"] for o in os_], g["n"])
    null_mean = float(np.mean([o["mean_z"] for o in os_]))
    print(f"[{name}] pixels {g['n']}: |z|>4 GPU {g['exceed']}, oracle nulls {[o['exceed'] for o in os_]} "
          f"(allowed {lim}); mean z GPU {g['mean_z']:+.4f}, nulls {null_mean:+.4f}; worst (row, col, |z|) "
          f"{[(i[0], i[1], round(float(zmax[i]), 2)) for i in idx]}")
    assert g["exceed"] <= lim, (name, g["exceed"], [o["exceed"] for o in os_], lim)
    if "blocks" in g:
        blim = allowed([o["block_exceed"] for o in os_], g["blocks"])
        print(f"[{name}] {block}x{block} blocks {g['blocks']}: |z|>4 GPU {g['block_exceed']}, nulls "
              f"{[o['block_exceed'] for o in os_]} (allowed {blim}); max |z| GPU {g['block_max']:.2f}, nulls "
              f"{max(o['block_max'] for o in os_):.2f}")
        assert g["block_exceed"] <= blim, (name, "blocks", g["block_exceed"], [o["block_exceed"] for o in os_], blim)
    sem = float(np.hypot(g["sem_z"], max(o["sem_z"] for o in os_)))
    assert abs(g["mean_z"] - null_mean) <= 4.0 * sem + 1e-3, (name, g["mean_z"], null_mean, sem)
    return g, os_


def gpu_moments(job, passes, crops):
    """Renders `passes` passes one at a time; returns per crop the sums and
    sums of squares of the per-pass colour samples (h, w, 3)."""
    prev = job.read_sums()[0]
    out = [[np.zeros(prev[y:y + h, x:x + w].shape), np.zeros(prev[y:y + h, x:x + w].shape)] for x, y, w, h in crops]
    for _ in range(passes):
        job.render_passes(1, sync=True)
        cur, _ = job.read_sums()
        sample = cur - prev
        prev = cur
        for (x, y, w, h), acc in zip(crops, out):
            s = sample[y:y + h, x:x + w]
            acc[0] += s
            acc[1] += s * s
    return out


def oracle_ref_and_null(ora, S, N, x, y, w, h, n_null=3):
    """The oracle's reference (N samples, passes S..S+N-1) and n_null null
    images (S samples each, on the passes after) for a window:
    (sums, sums of squares, [(null sums, null sums of squares), ...])."""
    r = ora.render(S, N, x, y, w, h)
    nulls = []
    for k in range(n_null):
        n = ora.render(S + N + k * S, S, x, y, w, h)
        nulls.append((n["color"], n["color_sq"]))
    return r["color"], r["color_sq"], nulls
