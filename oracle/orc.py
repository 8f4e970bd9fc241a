"""Python face of the oracle (test infrastructure only).

ctypes bindings to ``liborc.so`` (the C restatement in b2r_oracle.c) and to
``_ref/libheat_ref.so`` (the reference's own heat-3D.cpp, where built), plus
numpy restatements of the B2R subdomain bookkeeping:

* :func:`split_blocks` / :func:`join_blocks` -- a domain stored with an
  H-deep shell <-> Bx*By*Bz padded blocks of (B + 2H) cells per axis, the
  geometry of b2r.cpp:49-67 (``B2R_BLOCK_SIZE_* = B + 2*D*R``).
* :func:`halo_exchange` -- the X->Y->Z ordered face exchange of
  boundary_updating (b2r_halo_sync.cu:442-508) with the slab extents of
  sub_matrix_pack/unpack_{x,y,z} (b2r_halo_sync.cu:195-379): x slabs span the
  interior in y and z, y slabs the full padded x and interior z, z slabs the
  full padded x and y, so edges and corners arrive without diagonal messages.
  ``periodic`` wraps the neighbour index (new: the reference defines
  ``_PERIODIC_`` but never uses it, b2r_config.h:12).

Arrays are numpy with shape (nz, ny, nx) (x fastest), the reference layout.
Nothing here is on the product path.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_lib = None
_ref = None

_fp = C.POINTER(C.c_float)
_dp = C.POINTER(C.c_double)
_u8p = C.POINTER(C.c_uint8)


def lib():
    global _lib
    if _lib is None:
        from . import build as _b
        path = _b.build_oracle()
        L = C.CDLL(path)
        i, d = C.c_int, C.c_double
        L.orc_heat_substep_f32.argtypes = [_fp, _fp, i, i, i, i, d, d, d, d, i, i, i]
        L.orc_heat_substep_f64.argtypes = [_dp, _dp, i, i, i, i, d, d, d, d, i, i, i]
        L.orc_heat_run_f32.argtypes = [_fp, i, i, i, i, d, d, d, d, i, i, i]
        L.orc_heat_run_f64.argtypes = [_dp, i, i, i, i, d, d, d, d, i, i, i]
        L.orc_heat_cpu_main.argtypes = [_fp, i, i, i, i, i, d, d, d, d, i]
        L.orc_heat_cpu_main.restype = d
        L.orc_gol_substep.argtypes = [_u8p, _u8p, i, i, i, i, i, i]
        L.orc_gol_run_periodic.argtypes = [_u8p, i, i, i, i, i]
        L.orc_eqwp_ref_substep_f32.argtypes = [C.POINTER(_fp), i, i, i, i, i, i, i,
                                               i, i, i, i, i, d, i]
        L.orc_eqwp_ref_substep_f64.argtypes = [C.POINTER(_dp), i, i, i, i, i, i, i,
                                               i, i, i, i, i, d, i]
        L.orc_eqwp_stag_step_f32.argtypes = [C.POINTER(_fp), C.POINTER(_fp), i, i, i, d, d,
                                             i, i, i, i, i, i, d]
        L.orc_eqwp_stag_step_f64.argtypes = [C.POINTER(_dp), C.POINTER(_dp), i, i, i, d, d,
                                             i, i, i, i, i, i, d]
        L.orc_region.argtypes = [i, i, i, i, i, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.orc_eqwp_stag_adjoint_step_f64.argtypes = [C.POINTER(_dp), C.POINTER(_dp), C.POINTER(_dp),
                                                     C.POINTER(_dp), C.POINTER(_dp), i, i, i, d,
                                                     C.POINTER(C.c_int), C.POINTER(C.c_int)]
        _lib = L
    return _lib


def ref_lib():
    """The reference's own heat-3D.cpp (built on first use where its source
    tree is present), or None."""
    global _ref
    if _ref is None:
        path = os.path.join(HERE, "_ref", "libheat_ref.so")
        if not os.path.exists(path):
            from . import build as _b
            try:
                path = _b.build_ref() or path
            except Exception:
                return None
        if not os.path.exists(path):
            return None
        try:
            L = C.CDLL(path)
        except OSError:
            return None
        L.ref_heat_3D_cpu_main.argtypes = [_fp, C.c_int, C.c_int, C.c_int, C.c_int,
                                           C.c_int, C.c_int]
        L.ref_heat_3D_cpu_main.restype = C.c_float
        _ref = L
    return _ref


def _ptr(a, t):
    assert a.flags.c_contiguous
    return a.ctypes.data_as(t)


# ---------------------------------------------------------------- heat
REF_HEAT = dict(alpha_dt=0.1 * 0.1, dx=1.0, dy=1.0, dz=0.5)   # heat-3D.cpp:19-23


def heat_substep(a_in, a_out, D, i, H, edge, alpha_dt, dx, dy, dz):
    nz, ny, nx = a_in.shape
    if a_in.dtype == np.float32:
        lib().orc_heat_substep_f32(_ptr(a_in, _fp), _ptr(a_out, _fp), nx, ny, nz, D,
                                   alpha_dt, dx, dy, dz, i, H, edge)
    else:
        lib().orc_heat_substep_f64(_ptr(a_in, _dp), _ptr(a_out, _dp), nx, ny, nz, D,
                                   alpha_dt, dx, dy, dz, i, H, edge)


def heat_run(field, D, H, nsteps, alpha_dt, dx, dy, dz, nthreads=0):
    """nsteps steps over a domain with an H-deep fixed shell (in place)."""
    nz, ny, nx = field.shape
    if field.dtype == np.float32:
        lib().orc_heat_run_f32(_ptr(field, _fp), nx, ny, nz, D, alpha_dt, dx, dy, dz, H,
                               nsteps, nthreads)
    else:
        lib().orc_heat_run_f64(_ptr(field, _dp), nx, ny, nz, D, alpha_dt, dx, dy, dz, H,
                               nsteps, nthreads)
    return field


# central second-difference weights of order 2D (heat-3D.cu:15-28): centre,
# then distance 1, 2, ...
_LAP_W = {1: (-2.0, 1.0),
          2: (-5.0 / 2.0, 4.0 / 3.0, -1.0 / 12.0),
          3: (-49.0 / 18.0, 3.0 / 2.0, -3.0 / 20.0, 1.0 / 90.0),
          4: (-205.0 / 72.0, 8.0 / 5.0, -1.0 / 5.0, 8.0 / 315.0, -1.0 / 560.0)}


def heat_run_periodic(field, nsteps, alpha_dt, dx=1.0, dy=1.0, dz=1.0, D=1):
    """nsteps steps of radius D on a torus (every axis wraps), in float64:
    the update of heat-3D.cpp:57-60 / heat-3D.cu:228-231, u' = u + alpha_dt *
    (Lx/dx^2 + Ly/dy^2 + Lz/dz^2), L the order-2D central second difference
    (the weights of heat-3D.cu:15-28), its neighbour index wrapped (the
    reference defines no periodic heat; the wrap is this build's boundary
    option).  Returns a new float64 array."""
    w = _LAP_W[D]
    u = field.astype(np.float64)
    for _ in range(nsteps):
        lap = np.zeros_like(u)
        for ax, h in ((2, dx), (1, dy), (0, dz)):
            a = w[0] * u
            for k in range(1, D + 1):
                a = a + w[k] * (np.roll(u, k, axis=ax) + np.roll(u, -k, axis=ax))
            lap += a / (h * h)
        u = u + alpha_dt * lap
    return u


def heat_cpu_main(block, R, D, alpha_dt, dx, dy, dz, nthreads=0):
    nz, ny, nx = block.shape
    return lib().orc_heat_cpu_main(_ptr(block, _fp), R, D, nx, ny, nz, alpha_dt, dx, dy,
                                   dz, nthreads)


def ref_heat_cpu_main(block, R, nthreads=0):
    """heat_3D_cpu_main of the reference (delta1, its own constants)."""
    L = ref_lib()
    if L is None:
        raise RuntimeError("reference heat-3D.cpp was not built here")
    nz, ny, nx = block.shape
    return L.ref_heat_3D_cpu_main(_ptr(block, _fp), R, 1, nx, ny, nz, nthreads)


# ---------------------------------------------------------------- GoL
def gol_substep(a_in, a_out, i, H, edge):
    nz, ny, nx = a_in.shape
    lib().orc_gol_substep(_ptr(a_in, _u8p), _ptr(a_out, _u8p), nx, ny, nz, i, H, edge)


def gol_run_periodic(grid, nsteps, nthreads=0):
    nz, ny, nx = grid.shape
    lib().orc_gol_run_periodic(_ptr(grid, _u8p), nx, ny, nz, nsteps, nthreads)
    return grid


# ---------------------------------------------------------------- eqwp
def eqwp_ref_substep(fields, i, H, edge, ts, force):
    """fields: list of 10 arrays (vx..szz, disp); force: dict fy,fx0,fx1,fz0,fz1,fval,fsteps."""
    nz, ny, nx = fields[0].shape
    if fields[0].dtype == np.float32:
        arr = (_fp * 10)(*[_ptr(f, _fp) for f in fields])
        fn = lib().orc_eqwp_ref_substep_f32
    else:
        arr = (_dp * 10)(*[_ptr(f, _dp) for f in fields])
        fn = lib().orc_eqwp_ref_substep_f64
    fn(arr, nx, ny, nz, i, H, edge, ts, force["fy"], force["fx0"], force["fx1"],
       force["fz0"], force["fz1"], force["fval"], force["fsteps"])


def eqwp_stag_step(fields, mat, dt, dx, i, H, edge, src_xyz, src):
    nz, ny, nx = fields[0].shape
    if fields[0].dtype == np.float32:
        fa = (_fp * 9)(*[_ptr(f, _fp) for f in fields])
        ma = (_fp * 3)(*[_ptr(m, _fp) for m in mat])
        fn = lib().orc_eqwp_stag_step_f32
    else:
        fa = (_dp * 9)(*[_ptr(f, _dp) for f in fields])
        ma = (_dp * 3)(*[_ptr(m, _dp) for m in mat])
        fn = lib().orc_eqwp_stag_step_f64
    fn(fa, ma, nx, ny, nz, dt, dx, i, H, edge, src_xyz[0], src_xyz[1], src_xyz[2], src)


def eqwp_stag_run_periodic(fields, mat, dt, dx, amps, src_xyz):
    """len(amps) steps of the staggered FD4 scheme on a torus, in float64:
    the step of orc_eqwp_stag_step (b2r_oracle.c, no reference counterpart)
    with every neighbour index wrapped -- velocities from the stress
    divergence, then stresses from the new velocities, the source amplitude
    of the step added to sxx, syy and szz at src_xyz (x, y, z).  fields: vx,
    vy, vz, sxx, sxy, sxz, syy, syz, szz; mat: lambda, mu, buoyancy; arrays
    (nz, ny, nx).  Returns new float64 arrays."""
    c1, c2 = 9.0 / 8.0, -1.0 / 24.0
    f = [np.asarray(a, np.float64).copy() for a in fields]
    lam, mu, b = (np.asarray(a, np.float64) for a in mat)
    ax_of = {"x": 2, "y": 1, "z": 0}

    def sh(a, d, ax):          # a[i + d] along the axis
        return np.roll(a, -d, axis=ax_of[ax])

    def dp(a, ax):             # forward difference at i + 1/2
        return c1 * (sh(a, 1, ax) - a) + c2 * (sh(a, 2, ax) - sh(a, -1, ax))

    def dm(a, ax):             # backward difference at i - 1/2
        return c1 * (a - sh(a, -1, ax)) + c2 * (sh(a, 1, ax) - sh(a, -2, ax))

    vx, vy, vz, sxx, sxy, sxz, syy, syz, szz = range(9)
    x, y, z = src_xyz
    for amp in amps:
        a_x = dp(f[sxx], "x") + dm(f[sxy], "y") + dm(f[sxz], "z")
        a_y = dm(f[sxy], "x") + dp(f[syy], "y") + dm(f[syz], "z")
        a_z = dm(f[sxz], "x") + dm(f[syz], "y") + dp(f[szz], "z")
        f[vx] = f[vx] + dt * b * (a_x / dx)
        f[vy] = f[vy] + dt * b * (a_y / dx)
        f[vz] = f[vz] + dt * b * (a_z / dx)
        exx, eyy, ezz = dm(f[vx], "x") / dx, dm(f[vy], "y") / dx, dm(f[vz], "z") / dx
        l2m = lam + 2 * mu
        f[sxx] = f[sxx] + dt * (l2m * exx + lam * (eyy + ezz))
        f[syy] = f[syy] + dt * (l2m * eyy + lam * (exx + ezz))
        f[szz] = f[szz] + dt * (l2m * ezz + lam * (exx + eyy))
        f[sxy] = f[sxy] + dt * mu * ((dp(f[vx], "y") + dp(f[vy], "x")) / dx)
        f[sxz] = f[sxz] + dt * mu * ((dp(f[vx], "z") + dp(f[vz], "x")) / dx)
        f[syz] = f[syz] + dt * mu * ((dp(f[vy], "z") + dp(f[vz], "y")) / dx)
        for k in (sxx, syy, szz):
            f[k][z, y, x] += amp
    return f


# ---------------------------------------------------------------- B2R blocks
def edge_mask(b, nb, periodic=False):
    """Edge bit mask of block index b=(bx,by,bz) in a grid nb=(Bx,By,Bz)."""
    if periodic:
        return 0
    m = 0
    for a in range(3):
        if b[a] == 0:
            m |= 1 << (2 * a)
        if b[a] == nb[a] - 1:
            m |= 1 << (2 * a + 1)
    return m


def split_blocks(dom, nb, H, periodic=False):
    """Domain -> dict {(bx,by,bz): padded block}.

    Non-periodic: ``dom`` carries an H-deep shell, shape ENV + 2H per axis.
    Periodic: ``dom`` is the bare torus of shape ENV; halos wrap.
    """
    if periodic:
        dom = np.pad(dom, H, mode="wrap")
    env = [dom.shape[2 - a] - 2 * H for a in range(3)]
    bs = [env[a] // nb[a] for a in range(3)]
    assert all(bs[a] * nb[a] == env[a] for a in range(3))
    out = {}
    for bz in range(nb[2]):
        for by in range(nb[1]):
            for bx in range(nb[0]):
                z0, y0, x0 = bz * bs[2], by * bs[1], bx * bs[0]
                out[(bx, by, bz)] = np.ascontiguousarray(
                    dom[z0:z0 + bs[2] + 2 * H, y0:y0 + bs[1] + 2 * H, x0:x0 + bs[0] + 2 * H])
    return out


def join_blocks(blocks, nb, H, shell=None):
    """Padded blocks -> domain; interiors only, shell from ``shell`` (or 0)."""
    b0 = blocks[(0, 0, 0)]
    bs = [b0.shape[2 - a] - 2 * H for a in range(3)]
    env = [bs[a] * nb[a] for a in range(3)]
    if shell is None:
        dom = np.zeros((env[2], env[1], env[0]), b0.dtype)
        off = 0
    else:
        dom = shell.copy()
        off = H
    for (bx, by, bz), blk in blocks.items():
        dom[off + bz * bs[2]: off + (bz + 1) * bs[2],
            off + by * bs[1]: off + (by + 1) * bs[1],
            off + bx * bs[0]: off + (bx + 1) * bs[0]] = blk[H:H + bs[2], H:H + bs[1], H:H + bs[0]]
    return dom


def halo_exchange(blocks, nb, H, periodic=False):
    """X->Y->Z ordered halo exchange between resident blocks (in place)."""
    b0 = blocks[(0, 0, 0)]
    n = [b0.shape[2], b0.shape[1], b0.shape[0]]          # padded sizes x, y, z
    bs = [n[a] - 2 * H for a in range(3)]
    for axis in range(3):
        # extents of the slab on the other two axes (b2r_halo_sync.cu:203,235,267)
        ext = []
        for a in range(3):
            if a == axis:
                ext.append(None)
            elif a < axis:
                ext.append(slice(0, n[a]))               # already-exchanged axes: full
            else:
                ext.append(slice(H, H + bs[a]))          # later axes: interior only
        for key, blk in blocks.items():
            for side in (-1, 1):
                nbk = list(key)
                nbk[axis] += side
                if not (0 <= nbk[axis] < nb[axis]):
                    if not periodic:
                        continue
                    nbk[axis] %= nb[axis]
                src = blocks[tuple(nbk)]
                # my halo on `side` <- neighbour's interior slab facing me
                if side == -1:
                    dst_s, src_s = slice(0, H), slice(bs[axis], bs[axis] + H)
                else:
                    dst_s, src_s = slice(bs[axis] + H, bs[axis] + 2 * H), slice(H, 2 * H)
                d = [None, None, None]
                s = [None, None, None]
                for a in range(3):
                    d[a] = dst_s if a == axis else ext[a]
                    s[a] = src_s if a == axis else ext[a]
                blk[d[2], d[1], d[0]] = src[s[2], s[1], s[0]]
    return blocks


# ---------------------------------------------------------------- adjoint (FP64)
def eqwp_stag_adjoint_step(tmp, fv, fs, mat, g, k, lo, hi):
    """One reverse step of the discrete adjoint (orc_eqwp_stag_adjoint_step_f64)."""
    nz, ny, nx = tmp[0].shape
    P = lambda arrs: (_dp * len(arrs))(*[_ptr(a, _dp) for a in arrs])
    lib().orc_eqwp_stag_adjoint_step_f64(P(tmp), P(fv), P(fs), P(mat), P(g), nx, ny, nz, k,
                                         (C.c_int * 3)(*lo), (C.c_int * 3)(*hi))


def eqwp_stag_record(fields, mat, dt, dx, H, src_xyz, amps, rec, nsteps):
    """Forward nsteps (one block, fixed shell H); returns all states and vy at
    the receivers (rec: list of (x, y, z) block coordinates) after each step."""
    states = [[f.copy() for f in fields]]
    cur = [f.copy() for f in fields]
    d = np.zeros((nsteps, len(rec)), np.float64)
    for n in range(nsteps):
        eqwp_stag_step(cur, mat, dt, dx, 0, H, 63, src_xyz, float(amps[n]) if n < len(amps) else 0.0)
        for r, (x, y, z) in enumerate(rec):
            d[n, r] = cur[1][z, y, x]
        states.append([f.copy() for f in cur])
    return states, d


def eqwp_stag_gradient(fields, mat, dt, dx, H, src_xyz, amps, rec, nsteps, d_obs):
    """FP64 misfit J = 1/2 |d - d_obs|^2 and its gradient wrt lambda, mu, rho
    (full block arrays) by the discrete adjoint."""
    states, d = eqwp_stag_record(fields, mat, dt, dx, H, src_xyz, amps, rec, nsteps)
    res = d - d_obs
    J = 0.5 * float(np.sum(res * res))
    shape = fields[0].shape
    tmp = [np.zeros(shape) for _ in range(9)]      # vb(3), sb(6: xx xy xz yy yz zz)
    g = [np.zeros(shape) for _ in range(3)]
    lo = (H, H, H)
    hi = tuple(shape[2 - a] - 1 - H for a in range(3))
    sidx = [3, 4, 5, 6, 7, 8]                       # sxx sxy sxz syy syz szz in field order
    for n in range(nsteps - 1, -1, -1):
        for r, (x, y, z) in enumerate(rec):
            tmp[1][z, y, x] += res[n, r]
        fv = states[n + 1][:3]
        fs = [states[n][k] for k in sidx]
        eqwp_stag_adjoint_step(tmp, fv, fs, mat, g, dt / dx, lo, hi)
    g_rho = -g[2] * mat[2] ** 2
    return J, (g[0], g[1], g_rho), d, tmp


# ---------------------------------------------------------------- heat adjoint
# Differentiable heat step (new behaviour, no reference counterpart): the
# stencil of fdm_heat_diffuse_deltaD (heat-3D.cu:15-28, weights of
# heat-3D.cu:173-521) scaled per cell by a conductivity kappa,
#   u^{n+1} = u^n + kappa * L u^n  on the interior window [D, n-1-D] (one block,
# fixed shell), L u = w0 u + sum_k wx_k (u[x+k] + u[x-k]) + wy_k (...) + wz_k (...).
_HEAT_CW = [[0, 0, 0, 0, 0],
            [-2.0, 1.0, 0, 0, 0],
            [-5.0 / 2.0, 4.0 / 3.0, -1.0 / 12.0, 0, 0],
            [-49.0 / 18.0, 3.0 / 2.0, -3.0 / 20.0, 1.0 / 90.0, 0],
            [-205.0 / 72.0, 8.0 / 5.0, -1.0 / 5.0, 8.0 / 315.0, -1.0 / 560.0]]


def heat_lap_weights(D, alpha_dt, dx, dy, dz):
    """(w0, wx[D], wy[D], wz[D]): the weights rounded to FP32 as the GPU holds
    them, returned as FP64."""
    wx, wy, wz = alpha_dt / (dx * dx), alpha_dt / (dy * dy), alpha_dt / (dz * dz)
    f = lambda v: float(np.float32(v))
    cw = _HEAT_CW[D]
    return (f(cw[0] * (wx + wy + wz)), [f(wx * cw[k]) for k in range(1, D + 1)],
            [f(wy * cw[k]) for k in range(1, D + 1)], [f(wz * cw[k]) for k in range(1, D + 1)])


def heat_lap(u, D, w):
    """L u on the window [D, n-1-D] of every axis (FP64)."""
    w0, wx, wy, wz = w
    nz, ny, nx = u.shape
    c = (slice(D, nz - D), slice(D, ny - D), slice(D, nx - D))
    out = w0 * u[c]
    for k in range(1, D + 1):
        out = out + wx[k - 1] * (u[D:nz - D, D:ny - D, D + k:nx - D + k] + u[D:nz - D, D:ny - D, D - k:nx - D - k])
        out = out + wy[k - 1] * (u[D:nz - D, D + k:ny - D + k, D:nx - D] + u[D:nz - D, D - k:ny - D - k, D:nx - D])
        out = out + wz[k - 1] * (u[D + k:nz - D + k, D:ny - D, D:nx - D] + u[D - k:nz - D - k, D:ny - D, D:nx - D])
    return out


def heat_kappa_record(u0, kappa, D, w, rec, nsteps):
    """FP64 forward; rec: block coordinates (x, y, z).  (states, d[nsteps, nrec])."""
    u = np.asarray(u0, np.float64).copy()
    kap = np.asarray(kappa, np.float64)
    nz, ny, nx = u.shape
    c = (slice(D, nz - D), slice(D, ny - D), slice(D, nx - D))
    states = [u.copy()]
    d = np.zeros((nsteps, len(rec)))
    for n in range(nsteps):
        u[c] = u[c] + kap[c] * heat_lap(u, D, w)
        for r, (x, y, z) in enumerate(rec):
            d[n, r] = u[z, y, x]
        states.append(u.copy())
    return states, d


def heat_kappa_gradient(u0, kappa, D, w, rec, nsteps, d_obs):
    """FP64 misfit and dJ/dkappa (full block array, zero on the shell) by the
    discrete adjoint; also returns the adjoint of u^0."""
    states, d = heat_kappa_record(u0, kappa, D, w, rec, nsteps)
    res = d - d_obs
    J = 0.5 * float(np.sum(res * res))
    kap = np.asarray(kappa, np.float64)
    nz, ny, nx = kap.shape
    c = (slice(D, nz - D), slice(D, ny - D), slice(D, nx - D))
    lam = np.zeros(kap.shape)
    g = np.zeros(kap.shape)
    for n in range(nsteps - 1, -1, -1):
        for r, (x, y, z) in enumerate(rec):
            lam[z, y, x] += res[n, r]
        g[c] += lam[c] * heat_lap(states[n], D, w)
        y = np.zeros(kap.shape)
        y[c] = kap[c] * lam[c]
        lam[c] += heat_lap(y, D, w)
    return J, g, d, lam
