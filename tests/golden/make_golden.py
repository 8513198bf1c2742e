"""Generate the golden fixtures in tests/golden/ from an independent numpy restatement.

The reference (Java, PreibischLab/multiview-reconstruction) cannot run in this
environment and ships no deconvolution tests or vectors, so these fixtures come from
a second, independent restatement of its semantics written with numpy only (no code
shared with oracle/mvr_oracle.c):

* linear convolution: np.pad ('reflect' == imglib2 extendMirrorSingle, 'constant')
  followed by a full FFT convolution and the crop [k-1, k-1+b)
  (util/FFTConvolution.java:490-603, kernel centre at k/2);
* quotient / update / stats in numpy float32 arithmetic
  (DeconvolutionMethods.java:46-98, 103-182, 320-358, 370-419, 421);
* PSF preparation (DeconViewPSF.java:119-284, AdjustInput.java:52-122,
  Mirror.java:55-132);
* block grid, slab batches, deferred write-back
  (BlockGeneratorFixedSizePrecise.java:59-131, BlockSorter.java:55-143,
  MultiViewDeconvolutionSeq.java:57-180, MultiViewDeconvolutionMul.java:116-245).

Run:  python tests/golden/make_golden.py   (writes tests/golden/*.npz)
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "multiview-reconstruction_gb300"))
import synthetic  # noqa: E402

F32 = np.float32


# ----------------------------------------------------------------------------- conv
def np_convolve(block, kernel, mode, value=0.0):
    """mode: 'mirror' (mirror-single), 'value', 'zero'.  float64 result."""
    b = np.asarray(block, dtype=np.float64)
    k = np.asarray(kernel, dtype=np.float64)
    pads = []
    for d in range(3):
        kd = k.shape[d]
        c = kd // 2
        pads.append((kd - 1 - c, c))
    if mode == "mirror":
        # numpy 'reflect' cannot pad wider than n-1 in one go; repeat until done
        p = b
        rem = [list(x) for x in pads]
        while any(r[0] > 0 or r[1] > 0 for r in rem):
            step = []
            for d in range(3):
                n = p.shape[d]
                lo = min(rem[d][0], n - 1) if n > 1 else 0
                hi = min(rem[d][1], n - 1) if n > 1 else 0
                step.append((lo, hi))
            if all(s == (0, 0) for s in step):  # n == 1 along some axis: edge repeat
                step = [(r[0], r[1]) for r in rem]
                p = np.pad(p, step, mode="edge")
                break
            p = np.pad(p, step, mode="reflect")
            for d in range(3):
                rem[d][0] -= step[d][0]
                rem[d][1] -= step[d][1]
        padded = p
    elif mode == "value":
        padded = np.pad(b, pads, mode="constant", constant_values=value)
    else:
        padded = np.pad(b, pads, mode="constant", constant_values=0.0)
    s = [padded.shape[d] + k.shape[d] - 1 for d in range(3)]
    full = np.fft.irfftn(np.fft.rfftn(padded, s, axes=(0, 1, 2)) * np.fft.rfftn(k, s, axes=(0, 1, 2)), s, axes=(0, 1, 2))
    kz, ky, kx = k.shape
    bz, by, bx = b.shape
    return full[kz - 1:kz - 1 + bz, ky - 1:ky - 1 + by, kx - 1:kx - 1 + bx]


# ----------------------------------------------------------------------------- update
def tikhonov(v, lam):
    return (np.sqrt(1.0 + 2.0 * lam * v) - 1.0) / lam


def next_value_f32(last, integral, weight, lam, minI, maxI):
    last = last.astype(F32)
    value = (last * integral.astype(F32)).astype(F32)
    with np.errstate(invalid="ignore", divide="ignore", over="ignore"):
        if lam > 0:
            t = (tikhonov((value / F32(maxI)).astype(np.float64), lam)).astype(F32) * F32(maxI)
        else:
            t = value
        adjusted = np.where(value > 0, t, F32(minI)).astype(F32)
        nxt = np.where(np.isnan(adjusted), F32(minI), np.maximum(F32(minI), adjusted)).astype(F32)
        return (last + ((nxt - last) * weight.astype(F32))).astype(F32)


def next_value_f64(last, integral, weight, lam, minI, maxI):
    value = last * integral
    with np.errstate(invalid="ignore", divide="ignore", over="ignore"):
        t = tikhonov(value / maxI, lam) * maxI if lam > 0 else value
        adjusted = np.where(value > 0, t, minI)
        nxt = np.where(np.isnan(adjusted), minI, np.maximum(minI, adjusted))
    return last + (nxt - last) * weight


def block_seq(psi, img, w, k1, k2, lam, minI, maxI, fp64=False):
    if fp64:
        c1 = np_convolve(psi, k1, "mirror")
        with np.errstate(divide="ignore", invalid="ignore"):
            q = np.where(img > 0, img.astype(np.float64) / c1, 1.0)
        c2 = np_convolve(q, k2, "value", 1.0)
        nxt = next_value_f64(psi.astype(np.float64), c2, w.astype(np.float64), lam, float(F32(minI)),
                             float(F32(maxI)))
        ch = nxt - psi
        return nxt, (float(ch.sum()), float(max(-1.0, ch.max())))
    c1 = np_convolve(psi.astype(np.float64), k1, "mirror").astype(F32)
    with np.errstate(divide="ignore", invalid="ignore"):
        q = np.where(img > 0, (img.astype(F32) / c1).astype(F32), F32(1.0)).astype(F32)
    c2 = np_convolve(q.astype(np.float64), k2, "value", 1.0).astype(F32)
    nxt = next_value_f32(psi.astype(F32), c2, w, lam, minI, maxI)
    ch = (nxt - psi.astype(F32)).astype(F32)
    return nxt, (float(ch.astype(np.float64).sum()), float(max(-1.0, float(ch.max()))))


def block_mul(psi, imgs, ws, k1s, k2s, lam, minI, maxIs, fp64=False):
    nv = len(imgs)
    conv2 = []
    for v in range(nv):
        if fp64:
            c1 = np_convolve(psi, k1s[v], "mirror")
            with np.errstate(divide="ignore", invalid="ignore"):
                q = np.where(imgs[v] > 0, imgs[v].astype(np.float64) / c1, 1.0)
            conv2.append(np_convolve(q, k2s[v], "value", 1.0))
        else:
            c1 = np_convolve(psi.astype(np.float64), k1s[v], "mirror").astype(F32)
            with np.errstate(divide="ignore", invalid="ignore"):
                q = np.where(imgs[v] > 0, (imgs[v].astype(F32) / c1).astype(F32), F32(1.0)).astype(F32)
            conv2.append(np_convolve(q.astype(np.float64), k2s[v], "value", 1.0).astype(F32))
    miv = float(np.mean(np.asarray(maxIs, dtype=np.float64)))
    prod = np.ones(psi.shape, dtype=np.float64)
    sumw = np.zeros(psi.shape, dtype=np.float64)
    for v in range(nv):
        prod = prod * conv2[v].astype(np.float64)
        sumw = sumw + ws[v].astype(np.float64)
    prod = np.power(prod, 1.0 / nv)
    sumw = np.minimum(1.0, sumw)
    if fp64:
        nxt = next_value_f64(psi.astype(np.float64), prod, sumw, lam, float(F32(minI)), miv)
        ch = nxt - psi
        return nxt, (float(ch.sum()), float(max(-1.0, ch.max())))
    nxt = next_value_f32(psi.astype(F32), prod.astype(F32), sumw.astype(F32), lam, minI, F32(miv))
    ch = (nxt - psi.astype(F32)).astype(F32)
    return nxt, (float(ch.astype(np.float64).sum()), float(max(-1.0, float(ch.max()))))


# ----------------------------------------------------------------------------- PSF
def first_portion(size, T):
    if size <= T:
        npor = size
    else:
        npor = max(T, size // (64 * 64 * 64))
    chunk = size // npor
    while chunk == 0:
        npor -= 1
        chunk = size // npor
    return size if npor == 1 else chunk


def norm_to_sum1(k, T):
    flat = k.astype(np.float64).ravel()
    s = flat.sum()
    if T > 0:
        s += flat[:first_portion(flat.size, T)].sum()
    return (k.astype(np.float64) / s).astype(F32)


def invert(k):
    out = k.copy()
    for ax in range(3):  # axis in (x, y, z) order -> numpy axis 2, 1, 0
        npax = 2 - ax
        n = out.shape[npax]
        idx = np.arange(n)
        # Mirror.mirror: positions p <= n/2 swap with n-1-p, in iteration order
        perm = idx.copy()
        for p in range(n):
            if p <= n // 2:
                q = n - 1 - p
                perm[p], perm[q] = perm[q], perm[p]
        out = np.take(out, perm, axis=npax)
    return out


def conv_zero_f32(a, k):
    return np_convolve(a.astype(np.float64), k, "zero").astype(F32)


def psf_init(kernels, psf_type, T):
    """psf_type: 0 OPT_II, 1 OPT_I, 2 EFFICIENT_BAYESIAN, 3 INDEPENDENT"""
    k1 = [k.astype(F32).copy() for k in kernels]
    k2 = [None] * len(k1)
    nv = len(k1)
    for v in range(nv):
        k1[v] = norm_to_sum1(k1[v], T)
        if nv == 1 or psf_type == 3:
            k2[v] = invert(k1[v])
        elif psf_type == 2:
            tmp = invert(k1[v])
            for w in range(nv):
                if w == v:
                    continue
                o1 = conv_zero_f32(invert(k1[v]), k1[w])
                o2 = conv_zero_f32(o1, invert(k1[w]))
                tmp = (o2 * tmp).astype(F32)
            k2[v] = norm_to_sum1(tmp, T)
        elif psf_type == 1:
            tmp = k1[v].copy()
            for w in range(nv):
                if w == v:
                    continue
                o = conv_zero_f32(k1[v], invert(k1[w]))
                tmp = (o * tmp).astype(F32)
            k2[v] = invert(norm_to_sum1(tmp, T))
        else:
            e = k1[v].copy()
            for _ in range(1, nv):
                e = (e * k1[v]).astype(F32)
            k2[v] = invert(norm_to_sum1(e, T))
    return k1, k2


# ----------------------------------------------------------------------------- geometry / driver
def mirror_index(i, n):
    if n <= 1:
        return np.zeros_like(i)
    p = 2 * n - 2
    i = np.mod(i, p)
    return np.where(i >= n, p - i, i)


def blocks_for(D, k, bsize):
    kk = [2 * k[d] - 1 for d in range(3)]
    eff = [bsize[d] - kk[d] + 1 for d in range(3)]
    nb = [D[d] // eff[d] + (D[d] % eff[d] != 0) for d in range(3)]
    out = []
    for bz in range(nb[2]):
        for by in range(nb[1]):
            for bx in range(nb[0]):
                cb = (bx, by, bz)
                eo = [cb[d] * eff[d] for d in range(3)]
                es = [min(eff[d], D[d] - eo[d]) for d in range(3)]
                off = [eo[d] - kk[d] // 2 for d in range(3)]
                out.append(dict(off=off, eo=eo, es=es, loc=[kk[d] // 2 for d in range(3)]))
    sizes = []
    for d in range(3):
        s = 1
        for e in range(3):
            if e != d:
                s *= nb[e]
        sizes.append(s)
    key = {}
    for d in range(3):
        key[sizes[d]] = d
    srt = sorted(sizes)
    sd = None
    for i in range(3):
        if srt[i] >= 1 or i == 2:
            sd = key[srt[i]]
            break
    for bl in out:
        bl["batch"] = (bl["off"][sd] + kk[sd] // 2) // eff[sd]
    return out


def extract(vol, off, bsize, mirror):
    D = (vol.shape[2], vol.shape[1], vol.shape[0])
    idx = [np.arange(off[d], off[d] + bsize[d]) for d in range(3)]
    if mirror:
        ii = [mirror_index(idx[d], D[d]) for d in range(3)]
        return vol[np.ix_(ii[2], ii[1], ii[0])].copy()
    out = np.zeros((bsize[2], bsize[1], bsize[0]), dtype=vol.dtype)
    ok = [(idx[d] >= 0) & (idx[d] < D[d]) for d in range(3)]
    sub = vol[np.ix_(idx[2][ok[2]], idx[1][ok[1]], idx[0][ok[0]])]
    out[np.ix_(np.nonzero(ok[2])[0], np.nonzero(ok[1])[0], np.nonzero(ok[0])[0])] = sub
    return out


def paste(vol, bl, blk):
    eo, es, lo = bl["eo"], bl["es"], bl["loc"]
    vol[eo[2]:eo[2] + es[2], eo[1]:eo[1] + es[1], eo[0]:eo[0] + es[0]] = \
        blk[lo[2]:lo[2] + es[2], lo[1]:lo[1] + es[1], lo[0]:lo[0] + es[0]]


def decon_run(psi, imgs, ws, k1s, k2s, bsize, iters, mul, lam, minI, maxIs, fp64=False):
    psi = psi.astype(np.float64 if fp64 else F32).copy()
    D = (psi.shape[2], psi.shape[1], psi.shape[0])
    nv = len(imgs)
    steps = [0] if mul else list(range(nv))
    stats = []
    for _ in range(iters):
        for s in steps:
            kshape = (k1s[s].shape[2], k1s[s].shape[1], k1s[s].shape[0])
            bls = blocks_for(D, kshape, bsize)
            bls = [b for b in bls if np.any(extract(ws[s], b["off"], bsize, False) != 0)]
            nb = max(b["batch"] for b in bls) + 1
            single = len(bls) == 1
            prev = []
            ssum, smax = 0.0, -1.0
            for bt in range(nb):
                cur = []
                for bl in [b for b in bls if b["batch"] == bt]:
                    pb = extract(psi, bl["off"], bsize, True)
                    if mul:
                        ib = [extract(imgs[v], bl["off"], bsize, False) for v in range(nv)]
                        wb = [extract(ws[v], bl["off"], bsize, False) for v in range(nv)]
                        out, st = block_mul(pb, ib, wb, k1s, k2s, lam, minI, maxIs, fp64)
                    else:
                        ib = extract(imgs[s], bl["off"], bsize, False)
                        wb = extract(ws[s], bl["off"], bsize, False)
                        out, st = block_seq(pb, ib, wb, k1s[s], k2s[s], lam, minI, maxIs[s], fp64)
                    ssum += st[0]
                    smax = max(smax, st[1])
                    if single:
                        paste(psi, bl, out)
                    else:
                        cur.append((bl, out))
                if not single:
                    for bl, out in prev:
                        paste(psi, bl, out)
                    prev = cur
            for bl, out in prev:
                paste(psi, bl, out)
            stats.append((ssum, smax))
    return psi, np.array(stats)


def psi_init_avg(imgs):
    st = np.stack([i.astype(np.float64) for i in imgs])
    pos = st > 0
    cnt = pos.sum(0)
    mean = np.where(cnt > 0, np.where(pos, st, 0).sum(0) / np.maximum(cnt, 1), 0)
    avg = mean[cnt > 0].sum() / (cnt > 0).sum()
    mx = np.array([np.where(i > 0, i, 0).max() for i in imgs], dtype=F32)
    return avg, mx


def normalize_weights_hard(raw, osem=1.0):
    c = [np.minimum(1.0, r.astype(np.float64)) for r in raw]
    s = sum(c)
    out = []
    for v in range(len(raw)):
        my = c[v].astype(F32)
        r = np.where(s > 1, (my.astype(np.float64) / s).astype(F32), my).astype(np.float64)
        out.append(np.minimum(r * osem, 1.0).astype(F32))
    return out


# ----------------------------------------------------------------------------- fixtures
def main():
    rng = np.random.Generator(np.random.PCG64(7))
    out = {}
    # 1) convolution cases, all three extensions, odd and even kernel sizes
    blk = rng.uniform(0.5, 2.0, (9, 10, 11)).astype(F32)
    kodd = rng.uniform(0.0, 1.0, (5, 3, 7)).astype(F32)
    keven = rng.uniform(0.0, 1.0, (4, 3, 6)).astype(F32)
    np.savez_compressed(os.path.join(HERE, "conv_cases.npz"), block=blk, k_odd=kodd, k_even=keven,
                        mirror_odd=np_convolve(blk, kodd, "mirror"),
                        value_odd=np_convolve(blk, kodd, "value", 1.0),
                        zero_odd=np_convolve(blk, kodd, "zero"),
                        mirror_even=np_convolve(blk, keven, "mirror"),
                        value_even=np_convolve(blk, keven, "value", 1.0))

    # 2) small multiview dataset (2 views, 40x36x30, PSF 5x5x9 rotated 0/90)
    ds = synthetic.make_dataset((40, 36, 30), (0.0, 90.0), (5, 5, 9), n_beads=30, seed=11,
                                sigma_xy=1.0, sigma_z=2.0, weights="cosine")
    ws = normalize_weights_hard(ds.weights)
    avg, mx = psi_init_avg(ds.images)
    psi0 = np.full(ds.images[0].shape, F32(avg), dtype=F32)
    k1, k2 = psf_init(ds.psfs, 1, 4)
    # block case (whole block from the volume, as the driver would extract it)
    bsize = (24, 20, 28)
    bl = blocks_for((40, 36, 30), (5, 5, 9), bsize)[0]
    pb = extract(psi0 * rng.uniform(0.5, 1.5, psi0.shape).astype(F32), bl["off"], bsize, True)
    ib = [extract(ds.images[v], bl["off"], bsize, False) for v in range(2)]
    wb = [extract(ws[v], bl["off"], bsize, False) for v in range(2)]
    lam = 0.006
    s_out, s_st = block_seq(pb, ib[0], wb[0], k1[0], k2[0], lam, 1e-4, mx[0])
    s_out64, s_st64 = block_seq(pb, ib[0], wb[0], k1[0], k2[0], lam, 1e-4, mx[0], fp64=True)
    m_out, m_st = block_mul(pb, ib, wb, k1, k2, lam, 1e-4, mx)
    m_out64, m_st64 = block_mul(pb, ib, wb, k1, k2, lam, 1e-4, mx, fp64=True)
    np.savez_compressed(os.path.join(HERE, "block_cases.npz"), psi=pb, img0=ib[0], img1=ib[1],
                        w0=wb[0], w1=wb[1], k1_0=k1[0], k1_1=k1[1], k2_0=k2[0], k2_1=k2[1],
                        lam=lam, max=mx, seq_out=s_out, seq_stats=np.array(s_st), seq_out64=s_out64,
                        seq_stats64=np.array(s_st64), mul_out=m_out, mul_stats=np.array(m_st),
                        mul_out64=m_out64, mul_stats64=np.array(m_st64))

    # 3) whole-volume runs: block 28^3 on 40x36x30 with k = 5x5x9 (several blocks, 2 batches)
    seq_psi, seq_stats = decon_run(psi0, ds.images, ws, k1, k2, (28, 28, 28), 2, False, lam, 1e-4, mx)
    mul_psi, mul_stats = decon_run(psi0, ds.images, ws, k1, k2, (28, 28, 28), 2, True, lam, 1e-4, mx)
    seq_psi64, _ = decon_run(psi0, ds.images, ws, k1, k2, (28, 28, 28), 2, False, lam, 1e-4, mx, fp64=True)
    one_psi, one_stats = decon_run(psi0, ds.images, ws, k1, k2, (48, 44, 48), 2, False, 0.0, 1e-4, mx)
    np.savez_compressed(os.path.join(HERE, "volume_cases.npz"), img0=ds.images[0], img1=ds.images[1],
                        raw_w0=ds.weights[0], raw_w1=ds.weights[1], w0=ws[0], w1=ws[1],
                        psf0=ds.psfs[0], psf1=ds.psfs[1], k1_0=k1[0], k1_1=k1[1], k2_0=k2[0],
                        k2_1=k2[1], psi0=psi0, avg=avg, max=mx, lam=lam, seq_psi=seq_psi,
                        seq_stats=seq_stats, mul_psi=mul_psi, mul_stats=mul_stats, seq_psi64=seq_psi64,
                        one_psi=one_psi, one_stats=one_stats)

    # 4) PSF preparation, all four types, 3 views with different kernel sizes, T = 4
    psfs = [synthetic.make_psf((5, 5, 9), 1.0, 2.0, a) for a in (0.0, 45.0, 90.0)]
    psfs[2] = synthetic.make_psf((7, 5, 11), 1.0, 2.0, 90.0)
    res = {}
    for t in range(4):
        a, b = psf_init([p * 3.0 for p in psfs], t, 4)
        for v in range(3):
            res[f"t{t}_k1_{v}"] = a[v]
            res[f"t{t}_k2_{v}"] = b[v]
    evn = rng.uniform(0, 1, (4, 6, 3)).astype(F32)
    np.savez_compressed(os.path.join(HERE, "psf_cases.npz"), raw0=psfs[0] * 3.0, raw1=psfs[1] * 3.0,
                        raw2=psfs[2] * 3.0, even=evn, even_inv=invert(evn), **res)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
