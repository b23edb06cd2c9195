"""The schedule of the temporally blocked FP32 SOR kernel (poisson.cu, sor_tb_kernel), restated in numpy and
run on the CPU: checkerboard-packed arrays, tiles of rows x packed columns over every radial level with a halo
of 2S rows and S packed columns, 2S half-sweeps per pass on shrinking cones, the folded boundary cells written
by the cells two away from them, the periodic wrap of the packed columns, tile boundaries on even columns,
and passes that alternate between two pairs of packed arrays.

After N sweeps the tiled schedule must give the values of N plain red-black sweeps (the reference's update,
PressureSolver.h:318-495, with the boundary fold after each sweep, :718-746) to rounding. Every tile-local
index the kernel would touch is checked against the tile's extent, and every value a cell reads must have been
loaded (NaN marks the unloaded parts of a tile). The GPU tests in test_gpu_poisson.py compare the kernel itself
with the same reference."""
import numpy as np
import pytest

import poisson_ref as PR
from atsat_gb300 import synth
from helpers import case

LANES = 32
C43, C13 = 4.0 / 3.0, 1.0 / 3.0


def plain_sweeps(g, P, f, sweeps, omega=1.0):
    num1, num2, num3, den = PR.weights(g, P)
    im, jm, km = g.shape
    n = km - 1
    p = np.zeros(g.shape)
    ii, jj, kk = np.meshgrid(np.arange(1, im - 1), np.arange(1, jm - 1), np.arange(n), indexing="ij")
    for _ in range(sweeps):
        for colour in (0, 1):
            m = ((ii + jj + kk) & 1) == colour
            i, j, k = ii[m], jj[m], kk[m]
            kw, ke = (k - 1) % n, (k + 1) % n
            acc = (p[i + 1, j, k] + p[i - 1, j, k]) * num1[i, j] + (p[i, j + 1, k] + p[i, j - 1, k]) * num2[i, j] \
                + (p[i, j, ke] + p[i, j, kw]) * num3[i, j]
            p[i, j, k] = p[i, j, k] + omega * ((acc - f[i, j, k]) / den[i, j] - p[i, j, k])
        p[0] = C43 * p[1] - C13 * p[2]
        p[-1] = C43 * p[-2] - C13 * p[-3]
        p[:, 0] = C43 * p[:, 1] - C13 * p[:, 2]
        p[:, -1] = C43 * p[:, -2] - C13 * p[:, -3]
        p[:, :, -1] = p[:, :, 0]
    return p


def tiles(im, jm, km, S, blocks):
    """The host's tiling (plan_tb): packed columns in tiles of at most LANES - 2S starting on even columns,
    rows split evenly into at least two per tile, as many tiles as fill `blocks`."""
    nh, NJ = (km - 1) // 2, jm - 2
    ntm = (nh + LANES - 2 * S - 1) // (LANES - 2 * S)
    ntj = max(1, min(blocks // ntm, NJ // 2))
    out = []
    for t in range(ntm * ntj):
        tm, tj = t % ntm, t // ntm
        m0 = (tm * nh // ntm) & ~1
        m1 = nh if tm + 1 == ntm else ((tm + 1) * nh // ntm) & ~1
        out.append((m0, m1 - m0, 1 + tj * NJ // ntj, 1 + (tj + 1) * NJ // ntj))
    rj = (NJ + ntj - 1) // ntj + 4 * S
    return out, rj


def pack(x, im, jm, nh):
    """Pk[c][i, j, m] = x[i, j, 2 m + ((i + j + c) & 1)]"""
    i = np.arange(im)[:, None, None]
    j = np.arange(jm)[None, :, None]
    m = np.arange(nh)[None, None, :]
    return [x[i, j, 2 * m + ((i + j + c) & 1)] for c in (0, 1)]


def tiled_sweeps(g, P, f, sweeps, S=2, blocks=152, omega=1.0):
    num1, num2, num3, den = PR.weights(g, P)
    im, jm, km = g.shape
    n = km - 1
    nh = n // 2
    assert n % 4 == 0, "the tiled kernel runs on even half-rings"
    NI = im - 2
    tl, RJ = tiles(im, jm, km, S, blocks)
    A = pack(np.zeros(g.shape), im, jm, nh)
    F = pack(f, im, jm, nh)
    lanes = np.arange(LANES)
    done = 0
    while done < sweeps:
        ns = min(S, sweeps - done)
        done += ns
        B = [np.full_like(A[0], np.nan), np.full_like(A[0], np.nan)]
        for m0, TM, j0, j1 in tl:
            assert m0 % 2 == 0 and TM % 2 == 0 and 2 <= TM <= LANES - 2 * S and j1 - j0 >= 2
            assert j1 - j0 + 4 * S <= RJ
            jb = j0 - 2 * S
            gm = (m0 - S + lanes) % nh                      # the lanes' packed columns, wrapped
            sp = [np.full((im, RJ, LANES), np.nan) for _ in (0, 1)]
            rows = np.arange(RJ) + jb
            okr = (rows >= 0) & (rows < jm)
            okl = lanes < TM + 2 * S
            for c in (0, 1):
                blk = A[c][:, rows[okr], :][:, :, gm]
                sp[c][:, okr, :] = np.where(okl[None, None, :], blk, np.nan)
            for h in range(1, 2 * ns + 1):
                c, e = (h - 1) & 1, 2 * ns - h
                own, oth = sp[c], sp[1 - c]
                jlo, jhi = max(1, j0 - e), min(jm - 2, j1 - 1 + e)
                upd = {}
                for j in range(jlo, jhi + 1):
                    jj = j - jb
                    assert 1 <= jj <= RJ - 2
                    for i in range(1, NI + 1):
                        par = (i + j + c) & 1
                        kl = 2 * (lanes - S) + par
                        L = lanes[(kl >= -e) & (kl < 2 * TM + e)]
                        east, west = L + par, L - 1 + par
                        assert east.max() < LANES and west.min() >= 0
                        vals = [oth[i + 1, jj, L], oth[i - 1, jj, L], oth[i, jj + 1, L], oth[i, jj - 1, L],
                                oth[i, jj, east], oth[i, jj, west], own[i, jj, L]]
                        for v in vals:
                            assert not np.isnan(v).any(), ("read of an unloaded cell", i, j)
                        fv = F[c][i, j, gm[L]]
                        acc = (vals[0] + vals[1]) * num1[i, j] + (vals[2] + vals[3]) * num2[i, j] \
                            + (vals[4] + vals[5]) * num3[i, j]
                        old = vals[6]
                        pn = old + omega * ((acc - fv) / den[i, j] - old)
                        upd[(i, jj)] = (L, pn)
                        self_ = old if c == 0 else pn
                        if i == 2:
                            upd[(0, jj)] = (L, C43 * vals[1] - C13 * self_)
                        if i == im - 3:
                            upd[(im - 1, jj)] = (L, C43 * vals[0] - C13 * self_)
                        if j == 2 and jj >= 2:
                            upd[(i, jj - 2)] = (L, C43 * vals[3] - C13 * self_)
                        if j == jm - 3 and jj + 2 < RJ:
                            upd[(i, jj + 2)] = (L, C43 * vals[2] - C13 * self_)
                for (i, jj), (L, v) in upd.items():
                    own[i, jj, L] = v
            jsl = 0 if j0 == 1 else j0
            jsh = jm - 1 if j1 == jm - 1 else j1 - 1
            own_l = lanes[S:S + TM]
            for c in (0, 1):
                for j in range(jsl, jsh + 1):
                    blk = sp[c][:, j - jb, own_l]
                    assert not np.isnan(blk).any(), ("store of an unloaded cell", j)
                    assert np.isnan(B[c][:, j, m0:m0 + TM]).all(), "a cell written by two tiles"
                    B[c][:, j, m0:m0 + TM] = blk
        for c in (0, 1):
            assert not np.isnan(B[c]).any(), "a cell no tile wrote"
        A = B
    out = np.zeros(g.shape)
    i = np.arange(im)[:, None, None]
    j = np.arange(jm)[None, :, None]
    m = np.arange(nh)[None, None, :]
    for c in (0, 1):
        out[i, j, 2 * m + ((i + j + c) & 1)] = A[c]
    return out


@pytest.mark.parametrize("shape,blocks,sweeps", [((9, 13, 17), 152, 5), ((7, 30, 121), 20, 5), ((6, 16, 9), 152, 3)])
def test_tiled_schedule_equals_plain_sweeps(shape, blocks, sweeps):
    """One tile along phi with the halo wrapping past the ring (9 x 13 x 17, 6 x 16 x 9: a half-ring of 4
    packed columns, shorter than the tile's width), and three tiles along phi by six along theta
    (7 x 30 x 121); an odd sweep count, so the last pass has a single sweep."""
    g, P, _ = case(shape, seed=3)
    f = synth.poisson_source(g, seed=5)
    ref = plain_sweeps(g, P, f, sweeps)
    got = tiled_sweeps(g, P, f, sweeps, blocks=blocks)
    c = (slice(1, -1), slice(1, -1), slice(0, g.km - 1))
    err = np.max(np.abs(ref[c] - got[c])) / np.max(np.abs(ref[c]))
    assert err < 1e-13, err
