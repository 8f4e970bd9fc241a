"""The reference's own elastic-wave, Game-of-Life and heat CUDA kernels, run
as a second oracle.

TEST INFRASTRUCTURE ONLY: the GPU tests compare the library against these
kernels; nothing in the product loads them.

oracle/build.py compiles the reference's eqwp.cu (eqwp_fd4_stress and
eqwp_fd4_v{x,y,z}, eqwp.cu:60-477) unmodified into oracle/_ref/eqwp_ref.cubin
where the reference source tree is present; this module loads that cubin
through the CUDA driver API in the process's current (PyTorch) context and
drives it as eqwp_gpu_main does (eqwp.cu:661-688): per time step the stress
kernel, then vx, vy (with the displacement) and vz, on 16 x 16 thread blocks
over the padded block, R = 1; gol-3D.cu's gol_3d_kernel and heat-3D.cu's
fdm_heat_diffuse_delta1 likewise (run_reference_gol, run_reference_heat),
heat-3D.cu's fdm_heat_diffuse_delta2..4 from the cubins built at B2R_D = 2..4
(run_reference_heat_d) and its edge-flag kernel
fdm_heat_diffuse_delta1_verify at any R (run_reference_heat_verify).

The elastic-wave kernels are correct only inside their envelope: R = 1 and a block of at
most 16 rows (one thread-block tile in y) -- their y halo loads read row y-1
into the slot of row y-2 (eqwp.cu:118-123), which with a single y tile is
never executed.  run_reference refuses other shapes.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
CUBIN = os.path.join(HERE, "_ref", "eqwp_ref.cubin")
TILE = 16           # CUDA_BLOCK_SIZE (eqwp.cu:25)
FRC_TIME = 50       # eqwp.cu:14

# Itanium-mangled names of the reference's kernels (eqwp.cu:60,154,249,341)
_NAMES = {
    "stress": "_Z15eqwp_fd4_stressiiiPfS_S_S_S_S_S_S_S_i",
    "vx": "_Z11eqwp_fd4_vxiiiPfS_S_S_P6float3iii",
    "vy": "_Z11eqwp_fd4_vyiiiPfS_S_S_P6float3S_iii",
    "vz": "_Z11eqwp_fd4_vziiiPfS_S_S_P6float3iii",
}

GOL_CUBIN = os.path.join(HERE, "_ref", "gol_ref.cubin")
GOL_TILE = 32       # CUDA_BLOCK_SIZE (gol-3D.cu:8)
_GOL_NAME = "_Z13gol_3d_kernelPhS_iiii"   # gol_3d_kernel (gol-3D.cu:30)

HEAT_CUBIN = os.path.join(HERE, "_ref", "heat_ref.cubin")
HEAT_TILE = 32      # CUDA_BLOCK_SIZE (heat-3D.cu:8)
_HEAT_NAME = "_Z23fdm_heat_diffuse_delta1PfS_iiii"   # fdm_heat_diffuse_delta1 (heat-3D.cu:173)
# fdm_heat_diffuse_delta1_verify (heat-3D.cu:57): the edge-flag form of delta 1
_HEAT_VERIFY_NAME = "_Z30fdm_heat_diffuse_delta1_verifyPfS_iiiiiiii"
# fdm_heat_diffuse_delta2..4 (heat-3D.cu:250,337,432), one cubin per B2R_D
_HEAT_D_NAMES = {2: "_Z23fdm_heat_diffuse_delta2PfS_iiii", 3: "_Z23fdm_heat_diffuse_delta3PfS_iiii",
                 4: "_Z23fdm_heat_diffuse_delta4PfS_iiii"}


def heat_d_cubin(D):
    return HEAT_CUBIN if D == 1 else os.path.join(HERE, "_ref", f"heat_ref_d{D}.cubin")


_mods = {}


def available():
    return os.path.exists(CUBIN)


def gol_available():
    return os.path.exists(GOL_CUBIN)


def heat_available():
    return os.path.exists(HEAT_CUBIN)


def heat_d_available(D):
    return os.path.exists(heat_d_cubin(D))


def _driver():
    cu = C.CDLL("libcuda.so.1")
    cu.cuModuleLoadData.argtypes = [C.POINTER(C.c_void_p), C.c_void_p]
    cu.cuModuleGetFunction.argtypes = [C.POINTER(C.c_void_p), C.c_void_p, C.c_char_p]
    cu.cuLaunchKernel.argtypes = [C.c_void_p, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint,
                                  C.c_uint, C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]
    return cu


def _check(r, what):
    if r != 0:
        raise RuntimeError(f"{what} failed: CUresult {r}")


def _load(path, names):
    if path not in _mods:
        import torch
        torch.cuda.init()
        torch.zeros(1, device="cuda")          # the primary context is current on this thread
        cu = _driver()
        data = open(path, "rb").read()
        buf = C.create_string_buffer(data, len(data))
        mod = C.c_void_p()
        _check(cu.cuModuleLoadData(C.byref(mod), buf), "cuModuleLoadData")
        _mods[path] = (cu, mod, {}, buf)
    cu, mod, fns, _ = _mods[path]
    for k, name in names.items():      # functions of the module looked up on first use
        if k not in fns:
            f = C.c_void_p()
            _check(cu.cuModuleGetFunction(C.byref(f), mod, name.encode()), "cuModuleGetFunction " + k)
            fns[k] = f
    return _mods[path]


def _launch(cu, f, grid, stream, *args, tile=TILE):
    vals = []
    for a in args:
        vals.append(C.c_int(a) if isinstance(a, int) else C.c_void_p(a.data_ptr()))
    params = (C.c_void_p * len(vals))(*[C.cast(C.pointer(v), C.c_void_p) for v in vals])
    _check(cu.cuLaunchKernel(f, grid[0], grid[1], 1, tile, tile, 1, 0, stream, params, None), "cuLaunchKernel")


def reference_force(shape):
    """f_init of eqwp_cuda_init (eqwp.cu:561-566): Ngx*Ngz float3, y = -1e4
    on x in [Ngx/2, Ngx/2 + Ngx/10), z in [Ngz/2, Ngz/2 + Ngz/10)."""
    ngz, _, ngx = shape
    f = np.zeros((ngz, ngx, 3), np.float32)
    f[ngz // 2:ngz // 2 + ngz // 10, ngx // 2:ngx // 2 + ngx // 10, 1] = -10000.0
    return f


def run_reference(fields, nsteps, ts0=0):
    """fields: the 10 padded-block arrays (vx, vy, vz, sxx, sxy, sxz, syy, syz,
    szz, displacement), each (Ngz, Ngy, Ngx) float32.  Returns them after
    nsteps time steps of the reference kernels at R = 1."""
    import torch
    ngz, ngy, ngx = fields[0].shape
    if ngy > TILE:
        raise ValueError("the reference kernels are correct only within one %d-row tile in y" % TILE)
    cu, _, fns, _ = _load(CUBIN, _NAMES)
    dev = [torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda() for a in fields]
    vx, vy, vz, sxx, sxy, sxz, syy, syz, szz, disp = dev
    finit = torch.from_numpy(reference_force(fields[0].shape)).cuda()
    grid = ((ngx + TILE - 1) // TILE, (ngy + TILE - 1) // TILE)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    R = 1
    for n in range(nsteps):   # eqwp.cu:677-686 with b2r_i = 0
        ts = ts0 + n
        _launch(cu, fns["stress"], grid, stream, ngx, ngy, ngz, sxx, sxy, sxz, syy, syz, szz, vx, vy, vz, 0)
        _launch(cu, fns["vx"], grid, stream, ngx, ngy, ngz, vx, sxx, sxy, sxz, finit, ts, 0, R)
        _launch(cu, fns["vy"], grid, stream, ngx, ngy, ngz, vy, sxy, syy, syz, finit, disp, ts, 0, R)
        _launch(cu, fns["vz"], grid, stream, ngx, ngy, ngz, vz, sxz, syz, szz, finit, ts, 0, R)
    torch.cuda.synchronize()
    return [t.cpu().numpy() for t in dev]


def run_reference_gol(block, ngen):
    """block: (Ngz, Ngy, Ngx) uint8 with a one-cell fixed shell.  Returns it
    after ngen generations of the reference's gol_3d_kernel, one launch per
    generation into a copy of its input (gol-3D.cu:124-129: "no rule fires"
    keeps the cell), the shell restored after each one.  The kernel is
    correct only where one 32 x 32 tile covers the block in x and y: its
    behind/infront planes get no halo, and cells it does not update use an
    unset neighbour count (gol-3D.cu:49,76-91), which writes undefined values
    into the shell."""
    import torch
    ngz, ngy, ngx = block.shape
    if ngx > GOL_TILE or ngy > GOL_TILE:
        raise ValueError("the reference kernel is correct only within one %d x %d tile" % (GOL_TILE, GOL_TILE))
    cu, _, fns, _ = _load(GOL_CUBIN, {"gol": _GOL_NAME})
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    cur = torch.from_numpy(np.ascontiguousarray(block, np.uint8)).cuda()
    shell = torch.ones_like(cur, dtype=torch.bool)
    shell[1:-1, 1:-1, 1:-1] = False
    fixed = cur.clone()
    for _ in range(ngen):
        out = cur.clone()
        _launch(cu, fns["gol"], (1, 1), stream, cur, out, ngx, ngy, ngz, 0, tile=GOL_TILE)
        out[shell] = fixed[shell]
        cur = out
    torch.cuda.synchronize()
    return cur.cpu().numpy()


def run_reference_heat(block, nsteps):
    """block: (Ngz, Ngy, Ngx) float32 with a one-cell fixed shell.  Returns it
    after nsteps steps of the reference's fdm_heat_diffuse_delta1 at R = 1
    (its constants: alpha*dt = 0.01, dx = dy = 1, dz = 0.5, heat-3D.cu:9-13),
    driven as heat_3D_gpu_main drives it (heat-3D.cu:583-642): both device
    buffers start as the block, 32 x 32 thread blocks, ping-pong."""
    import torch
    ngz, ngy, ngx = block.shape
    cu, _, fns, _ = _load(HEAT_CUBIN, {"heat": _HEAT_NAME})
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    a = torch.from_numpy(np.ascontiguousarray(block, np.float32)).cuda()
    b = a.clone()
    grid = ((ngx + HEAT_TILE - 1) // HEAT_TILE, (ngy + HEAT_TILE - 1) // HEAT_TILE)
    for _ in range(nsteps):
        _launch(cu, fns["heat"], grid, stream, a, b, ngx, ngy, ngz, 0, tile=HEAT_TILE)
        a, b = b, a
    torch.cuda.synchronize()
    return a.cpu().numpy()


def heat_d_envelope(shape, D):
    """Whether fdm_heat_diffuse_delta<D> is correct on a (Ngz, Ngy, Ngx) block
    at R = 1: one 32-row tile in y (its y halo loads read row y-1 into the
    slot of row y-D, heat-3D.cu:304-309), and in x every thread that loads a
    left halo of the last x tile updates its own cell (the loads sit under
    the update test, heat-3D.cu:298-303) -- (Ngx-1-D) mod 32 >= D-1 -- or a
    single x tile."""
    ngz, ngy, ngx = shape
    if ngy > HEAT_TILE:
        return False
    return ngx <= HEAT_TILE or (ngx - 1 - D) % HEAT_TILE >= D - 1


def run_reference_heat_d(block, D, nsteps):
    """block: (Ngz, Ngy, Ngx) float32 with a D-cell fixed shell.  Returns it
    after nsteps steps of the reference's fdm_heat_diffuse_delta<D> (D = 2,
    3, 4; 1 runs the delta-1 kernel) at R = 1 with its constants
    (alpha*dt = 0.01, dx = dy = 1, dz = 0.5, heat-3D.cu:9-13), driven as
    heat_3D_gpu_main drives it (heat-3D.cu:583-628): both device buffers
    start as the block, 32 x 32 thread blocks, ping-pong.  Refuses blocks
    outside the kernel's correct envelope (heat_d_envelope)."""
    import torch
    if D == 1:
        return run_reference_heat(block, nsteps)
    ngz, ngy, ngx = block.shape
    if not heat_d_envelope(block.shape, D):
        raise ValueError("fdm_heat_diffuse_delta%d is correct only within one 32-row y tile, "
                         "with (Ngx-1-D) mod 32 >= D-1" % D)
    cu, _, fns, _ = _load(heat_d_cubin(D), {"heat": _HEAT_D_NAMES[D]})
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    a = torch.from_numpy(np.ascontiguousarray(block, np.float32)).cuda()
    b = a.clone()
    grid = ((ngx + HEAT_TILE - 1) // HEAT_TILE, (ngy + HEAT_TILE - 1) // HEAT_TILE)
    for _ in range(nsteps):
        _launch(cu, fns["heat"], grid, stream, a, b, ngx, ngy, ngz, 0, tile=HEAT_TILE)
        a, b = b, a
    torch.cuda.synchronize()
    return a.cpu().numpy()


def run_reference_heat_verify(block, R, ef):
    """heat_3D_gpu_main (heat-3D.cu:583-637) with the edge-flag kernel it
    keeps commented out (fdm_heat_diffuse_delta1_verify, heat-3D.cu:57-158,
    606): both device buffers start as the (Ngz, Ngy, Ngx) float32 block, R
    ping-pong launches with b2r_i = 0..R-1 and ef = (xef, yef, zef) in
    {-1, 0, 1}, then planes [R, Ngz-R) of the result replace the block's.
    Any number of 32 x 32 tiles: the radius-1 halo loads are right."""
    import torch
    ngz, ngy, ngx = block.shape
    cu, _, fns, _ = _load(HEAT_CUBIN, {"heat": _HEAT_NAME, "verify": _HEAT_VERIFY_NAME})
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    a = torch.from_numpy(np.ascontiguousarray(block, np.float32)).cuda()
    b = a.clone()
    grid = ((ngx + HEAT_TILE - 1) // HEAT_TILE, (ngy + HEAT_TILE - 1) // HEAT_TILE)
    for i in range(R):
        _launch(cu, fns["verify"], grid, stream, a, b, ngx, ngy, ngz, i, int(ef[0]), int(ef[1]), int(ef[2]), R,
                tile=HEAT_TILE)
        a, b = b, a
    torch.cuda.synchronize()
    out = np.array(block, np.float32, copy=True)
    out[R:ngz - R] = a.cpu().numpy()[R:ngz - R]
    return out


def time_reference_heat(block, nsteps, reps=3):
    """Milliseconds per run of nsteps reference delta-1 steps on the device
    (CUDA events, after one untimed run), the block resident in HBM."""
    import torch
    ngz, ngy, ngx = block.shape
    cu, _, fns, _ = _load(HEAT_CUBIN, {"heat": _HEAT_NAME})
    s = torch.cuda.current_stream()
    stream = C.c_void_p(s.cuda_stream)
    a = torch.from_numpy(np.ascontiguousarray(block, np.float32)).cuda()
    b = a.clone()
    grid = ((ngx + HEAT_TILE - 1) // HEAT_TILE, (ngy + HEAT_TILE - 1) // HEAT_TILE)

    def run():
        x, y = a, b
        for _ in range(nsteps):
            _launch(cu, fns["heat"], grid, stream, x, y, ngx, ngy, ngz, 0, tile=HEAT_TILE)
            x, y = y, x

    run()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(reps):
        run()
    e1.record(s)
    e1.synchronize()
    return e0.elapsed_time(e1) / reps


def time_reference_eqwp(shape, nsteps, reps=1):
    """Milliseconds per run of nsteps reference elastic-wave steps (stress,
    vx, vy, vz per step) on a zero block of the given (Ngz, Ngy, Ngx) shape
    with the body force, fields resident (CUDA events, after one untimed
    run).  Timing only: beyond one 16-row tile in y the kernels' results are
    wrong at tile edges (eqwp.cu:118-123), their memory accesses stay inside
    the block."""
    import torch
    ngz, ngy, ngx = shape
    cu, _, fns, _ = _load(CUBIN, _NAMES)
    s = torch.cuda.current_stream()
    stream = C.c_void_p(s.cuda_stream)
    f = [torch.zeros(shape, dtype=torch.float32, device="cuda") for _ in range(10)]
    vx, vy, vz, sxx, sxy, sxz, syy, syz, szz, disp = f
    finit = torch.from_numpy(reference_force(shape)).cuda()
    grid = ((ngx + TILE - 1) // TILE, (ngy + TILE - 1) // TILE)

    def run():
        for ts in range(nsteps):
            _launch(cu, fns["stress"], grid, stream, ngx, ngy, ngz, sxx, sxy, sxz, syy, syz, szz, vx, vy, vz, 0)
            _launch(cu, fns["vx"], grid, stream, ngx, ngy, ngz, vx, sxx, sxy, sxz, finit, ts, 0, 1)
            _launch(cu, fns["vy"], grid, stream, ngx, ngy, ngz, vy, sxy, syy, syz, finit, disp, ts, 0, 1)
            _launch(cu, fns["vz"], grid, stream, ngx, ngy, ngz, vz, sxz, syz, szz, finit, ts, 0, 1)

    run()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(reps):
        run()
    e1.record(s)
    e1.synchronize()
    return e0.elapsed_time(e1) / reps


def time_reference_gol(shape, ngen, reps=1):
    """Milliseconds per run of ngen launches of the reference's
    gol_3d_kernel on a random (Ngz, Ngy, Ngx) block, ping-pong as
    gol_3D_gpu_main runs it (gol-3D.cu:124-145), resident (CUDA events,
    after one untimed run).  Timing only: beyond one 32 x 32 tile its results
    are wrong at tile edges; its memory accesses stay inside the block."""
    import torch
    ngz, ngy, ngx = shape
    cu, _, fns, _ = _load(GOL_CUBIN, {"gol": _GOL_NAME})
    s = torch.cuda.current_stream()
    stream = C.c_void_p(s.cuda_stream)
    a = (torch.rand(shape, device="cuda") < 0.3).to(torch.uint8)
    b = a.clone()
    grid = ((ngx + GOL_TILE - 1) // GOL_TILE, (ngy + GOL_TILE - 1) // GOL_TILE)

    def run():
        x, y = a, b
        for _ in range(ngen):
            _launch(cu, fns["gol"], grid, stream, x, y, ngx, ngy, ngz, 0, tile=GOL_TILE)
            x, y = y, x

    run()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(reps):
        run()
    e1.record(s)
    e1.synchronize()
    return e0.elapsed_time(e1) / reps

