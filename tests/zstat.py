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
for a null image: S further oracle samples per pixel on a third set of
streams, against the same reference. The GPU image passes when its
exceedance count is within the 99.9% Poisson bound of an expectation equal
to the null's count (or the Gaussian expectation, when larger); the same
holds on 8x8-pixel blocks, and the mean z (bias) must match the null's to 4
standard errors. Counts are printed for both.
"""
from __future__ import annotations

import numpy as np

P_EXCEED_4SIGMA = 6.334248366623996e-05   # 2 (1 - Phi(4))


def poisson_bound(expected: float, q: float = 0.999) -> int:
    """Smallest k with P(X <= k) >= q for X ~ Poisson(expected)."""
    k, term = 0, np.exp(-expected)
    cdf = term
    while cdf < q:
        k += 1
        term *= expected / k
        cdf += term
    return k


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
    exceed = int((np.abs(z) > 4.0).sum())
    zf = z[np.isfinite(z)]
    out = {"n": z.size, "exceed": exceed, "mean_z": float(zf.mean()), "sem_z": float(zf.std() / np.sqrt(zf.size))}
    if z.shape[0] >= block and z.shape[1] >= block:
        bd, bv = _blocks(d, block), _blocks(var_mean, block)
        zb = bd / np.sqrt(np.maximum(bv, 1e-300))
        zb = np.where(np.abs(bd) <= 1e-6 * (1.0 + np.abs(_blocks(mc, block))), 0.0, zb)
        out.update(blocks=zb.size, block_exceed=int((np.abs(zb) > 4.0).sum()), block_max=float(np.abs(zb).max()))
    return out


def allowed(null_count: int, n: int) -> int:
    """Exceedances allowed when the null image had null_count: the 99.9%
    Poisson bound of an expected count equal to the null's (or the Gaussian
    expectation n * 6.3e-5 when that is larger)."""
    return poisson_bound(max(float(null_count), n * P_EXCEED_4SIGMA))


def ztest(name, ts, ts2, S, cs, cs2, N, ns, ns2, block=8):
    """ts/ts2: the test image's per-pixel sums and sums of squares of S
    samples; cs/cs2: the oracle reference's, N samples; ns/ns2: the oracle
    null image's, S samples (streams disjoint from the other two)."""
    z, d, vm, mc = _z(ts, ts2, S, cs, cs2, N)
    z0, d0, vm0, _ = _z(ns, ns2, S, cs, cs2, N)
    g, o = _counts(z, d, vm, mc, block), _counts(z0, d0, vm0, mc, block)
    worst = np.argsort(-np.abs(z).ravel())[:4]
    idx = [tuple(int(i) for i in np.unravel_index(k, z.shape)) for k in worst]
    lim = allowed(o["exceed"], g["n"])
    print(f"[{name}] pixel-channels {g['n']}: |z|>4 GPU {g['exceed']}, oracle null {o['exceed']} (allowed {lim}); "
          f"mean z GPU {g['mean_z']:+.4f}, null {o['mean_z']:+.4f}; worst (row, col, ch, z) "
          f"{[(i[0], i[1], i[2], round(float(z[i]), 2)) for i in idx]}")
    assert g["exceed"] <= lim, (name, g["exceed"], o["exceed"], lim)
    if "blocks" in g:
        blim = allowed(o["block_exceed"], g["blocks"])
        print(f"[{name}] {block}x{block} blocks x channels {g['blocks']}: |z|>4 GPU {g['block_exceed']}, "
              f"null {o['block_exceed']} (allowed {blim}); max |z| GPU {g['block_max']:.2f}, null {o['block_max']:.2f}")
        assert g["block_exceed"] <= blim, (name, "blocks", g["block_exceed"], o["block_exceed"], blim)
    sem = np.hypot(g["sem_z"], o["sem_z"])
    assert abs(g["mean_z"] - o["mean_z"]) <= 4.0 * sem + 1e-3, (name, g["mean_z"], o["mean_z"], sem)
    return g, o


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


def oracle_ref_and_null(ora, S, N, x, y, w, h):
    """The oracle's reference (N samples, passes S..S+N-1) and null image (S
    samples, passes S+N..S+N+S-1) for a window: (sums, sums of squares) each."""
    r = ora.render(S, N, x, y, w, h)
    n = ora.render(S + N, S, x, y, w, h)
    return r["color"], r["color_sq"], n["color"], n["color_sq"]
