"""CPU model of the index arithmetic of the domain <-> blocks row kernels
(halo.cu scatter_kernel / gather_kernel): every (row, lane, unroll slot)
access is checked against its buffer and its row, and the result compared
with the plain per-cell mapping (domain cell of every block cell; owner
block of every domain cell).  The kernels' own results are checked on the
GPU by every upload/download test; this pins the arithmetic, including the
layouts that run first on new shapes, without one."""
import itertools

import numpy as np
import pytest

U, W = 4, 32     # kRowUnroll, lanes per warp (halo.cu)


def roundup(v, a):
    return (v + a - 1) // a * a


def layout(env, blocks, H, cb, periodic):
    B = [e // b for e, b in zip(env, blocks)]
    n = [b + 2 * H for b in B]
    A, m = 128 // cb, 16 // cb
    xoff = roundup(H + m, A) - H
    P = roundup(xoff + n[0] + 2 * m, A)
    plane = P * n[1]
    bstride = plane * n[2]
    return dict(n=n, B=B, nb=list(blocks), nblk=blocks[0] * blocks[1] * blocks[2], H=H, xoff=xoff, P=P,
                plane=plane, bstride=bstride, periodic=periodic)


def wrap_once(g, e):
    return g + e if g < 0 else (g - e if g >= e else g)


def scatter_model(dom, L, shell):
    """scatter_kernel, warp row by warp row."""
    n, B, nb, H = L["n"], L["B"], L["nb"], L["H"]
    e0, e1, e2 = nb[0] * B[0], nb[1] * B[1], nb[2] * B[2]
    dn0, dn1 = e0 + 2 * shell, e1 + 2 * shell
    out = np.full(L["bstride"] * L["nblk"], -7, np.int64)
    nrows = n[1] * n[2] * L["nblk"]
    for r in range(nrows):
        y = r % n[1]; rz = r // n[1]; z = rz % n[2]; blk = rz // n[2]
        b0 = blk % nb[0]; b1 = (blk // nb[0]) % nb[1]; b2 = blk // (nb[0] * nb[1])
        gx0 = b0 * B[0] - H
        g1 = b1 * B[1] + y - H; g2 = b2 * B[2] + z - H
        row = -1
        if L["periodic"]:
            g1 = wrap_once(g1, e1); g2 = wrap_once(g2, e2)
            if 0 <= g1 < e1 and 0 <= g2 < e2:
                row = (g2 * e1 + g1) * e0
        elif -shell <= g1 < e1 + shell and -shell <= g2 < e2 + shell:
            row = ((g2 + shell) * dn1 + (g1 + shell)) * dn0 + shell
        o = blk * L["bstride"] + z * L["plane"] + y * L["P"] + L["xoff"]
        for xb in range(0, n[0], W * U):
            for u in range(U):
                for lane in range(W):
                    x = xb + u * W + lane
                    g0 = gx0 + x
                    if L["periodic"]:
                        g0 = wrap_once(g0, e0); ok = 0 <= g0 < e0
                    else:
                        ok = -shell <= g0 < e0 + shell
                    if row >= 0 and x < n[0] and ok:
                        idx = row + g0
                        assert 0 <= idx < dom.size, ("scatter read", idx)
                        v = dom[idx]
                    else:
                        v = 0
                    if x < n[0]:
                        assert 0 <= o + x < out.size and L["xoff"] <= (o + x) % L["P"] < L["xoff"] + n[0]
                        out[o + x] = v
    return out


def scatter_ref(dom, L, shell):
    """The previous kernel's mapping, cell by cell."""
    n, B, nb, H = L["n"], L["B"], L["nb"], L["H"]
    dn = [nb[a] * B[a] + 2 * shell for a in range(3)]
    out = np.full(L["bstride"] * L["nblk"], -7, np.int64)
    for blk in range(L["nblk"]):
        b = [blk % nb[0], (blk // nb[0]) % nb[1], blk // (nb[0] * nb[1])]
        for z, y, x in itertools.product(range(n[2]), range(n[1]), range(n[0])):
            g = [b[0] * B[0] + x - H, b[1] * B[1] + y - H, b[2] * B[2] + z - H]
            if L["periodic"]:
                e = [nb[a] * B[a] for a in range(3)]
                g = [((g[a] % e[a]) + e[a]) % e[a] for a in range(3)]
                v = dom[(g[2] * e[1] + g[1]) * e[0] + g[0]]
            else:
                g = [g[a] + shell for a in range(3)]
                v = dom[(g[2] * dn[1] + g[1]) * dn[0] + g[0]] if all(0 <= g[a] < dn[a] for a in range(3)) else 0
            out[blk * L["bstride"] + z * L["plane"] + y * L["P"] + L["xoff"] + x] = v
    return out


def owner_of(g, B, nb):
    b = g // B if g >= 0 else 0
    return nb - 1 if b >= nb else b


def gather_model(blocks, L, shell):
    """gather_kernel, warp row by warp row, x-block segment by segment."""
    n, B, nb, H = L["n"], L["B"], L["nb"], L["H"]
    dn0, dn1, dn2 = nb[0] * B[0] + 2 * shell, nb[1] * B[1] + 2 * shell, nb[2] * B[2] + 2 * shell
    dom = np.full(dn0 * dn1 * dn2, -9, np.int64)
    for r in range(dn1 * dn2):
        g1 = r % dn1 - shell; g2 = r // dn1 - shell
        bb1, bb2 = owner_of(g1, B[1], nb[1]), owner_of(g2, B[2], nb[2])
        l1, l2 = g1 - bb1 * B[1] + H, g2 - bb2 * B[2] + H
        assert 0 <= l1 < n[1] and 0 <= l2 < n[2]
        drow = r * dn0
        o = l2 * L["plane"] + l1 * L["P"] + L["xoff"]
        blk_yz = nb[0] * (bb1 + nb[1] * bb2)
        for bb0 in range(nb[0]):
            lo = 0 if bb0 == 0 else shell + bb0 * B[0]
            hi = dn0 if bb0 == nb[0] - 1 else shell + (bb0 + 1) * B[0]
            srow = (blk_yz + bb0) * L["bstride"] + o + (H - shell - bb0 * B[0])
            for xb in range(lo, hi, W * U):
                for u in range(U):
                    for lane in range(W):
                        d0 = xb + u * W + lane
                        if d0 < hi:
                            idx = srow + d0
                            assert 0 <= idx < blocks.size, ("gather read", idx)
                            lx = idx - (blk_yz + bb0) * L["bstride"] - o
                            assert 0 <= lx < n[0], ("gather x", lx)
                            assert 0 <= drow + d0 < dom.size
                            dom[drow + d0] = blocks[idx]
    return dom


def gather_ref(blocks, L, shell):
    n, B, nb, H = L["n"], L["B"], L["nb"], L["H"]
    dn = [nb[a] * B[a] + 2 * shell for a in range(3)]
    dom = np.full(dn[0] * dn[1] * dn[2], -9, np.int64)
    for e in range(dom.size):
        d0 = e % dn[0]; r = e // dn[0]; d1 = r % dn[1]; d2 = r // dn[1]
        g = [d0 - shell, d1 - shell, d2 - shell]
        b, l = [], []
        for a in range(3):
            bb = g[a] // B[a] if g[a] >= 0 else -1
            bb = 0 if bb < 0 else (nb[a] - 1 if bb >= nb[a] else bb)
            b.append(bb); l.append(g[a] - bb * B[a] + H)
        blk = b[0] + nb[0] * (b[1] + nb[1] * b[2])
        dom[e] = blocks[blk * L["bstride"] + l[2] * L["plane"] + l[1] * L["P"] + L["xoff"] + l[0]]
    return dom

CASES = [
    # env, blocks, halo H, shell, cell bytes, periodic
    ((20, 12, 10), (1, 1, 1), 1, 1, 4, 0),
    ((20, 12, 10), (2, 1, 2), 3, 1, 4, 0),     # heat R = 3
    ((24, 16, 12), (2, 2, 1), 4, 2, 4, 0),     # elastic wave: H = 4R, shell 2
    ((30, 12, 16), (3, 2, 2), 4, 4, 4, 0),     # heat D = 4
    ((16, 16, 16), (2, 2, 2), 4, 0, 1, 1),     # Game of Life torus, R = 4
    ((8, 8, 8), (1, 1, 1), 4, 0, 1, 1),        # halo of half a block, one block per axis
    ((10, 8, 6), (2, 1, 2), 3, 0, 4, 1),       # halo as deep as a block
    ((130, 6, 5), (1, 1, 1), 2, 1, 4, 0),      # rows longer than one 128-cell sweep
    ((33, 7, 9), (1, 1, 1), 1, 1, 1, 0),       # byte cells with a shell
]


@pytest.mark.parametrize("env,blocks,H,shell,cb,per", CASES)

def test_row_copy_index_model(env, blocks, H, shell, cb, per):
    L = layout(env, blocks, H, cb, per)
    dn = [e + 2 * shell for e in env]
    rng = np.random.default_rng(0)
    dom = rng.integers(1, 1 << 30, dn[0] * dn[1] * dn[2])
    assert np.array_equal(scatter_model(dom, L, shell), scatter_ref(dom, L, shell))
    blocks_arr = rng.integers(1, 1 << 30, L["bstride"] * L["nblk"])
    got = gather_model(blocks_arr, L, shell)
    assert np.array_equal(got, gather_ref(blocks_arr, L, shell))
    assert (got != -9).all()
