"""b2r_gb300 -- the B2R stencil hot path on one GB300, host side.

A thin Python face over the C ABI of ``libb2r.so`` (include/b2r.h), shaped
like the reference's entry points (b2r.cpp, heat-3D.cu, gol-3D.cu, eqwp.cu,
b2r_halo_sync.cu):

* :class:`Domain` -- one b2r handle: the Bx*By*Bz subdomains of a global
  domain resident on the GPU (``simu_env_init`` + ``b2r_sync_init`` +
  ``eqwp_cuda_init``), ``step`` = the main loop of b2r.cpp:179-221
  (halo exchange every R steps, then R model steps), ``boundary_updating``
  and ``boundary_updating_direct`` as in b2r_halo_sync.cu.
* :func:`heat_3D_gpu_main`, :func:`gol_3D_gpu_main` -- the per-block entries
  of heat-3D.cu:583 and gol-3D.cu:119 on a host numpy block.

All compute runs in the CUDA library; there is no CPU fallback.  Importing
this package without a built ``libb2r.so`` raises.
"""
import ctypes as C
import os

import numpy as np

__all__ = ["Domain", "Batch", "EqwpBatch", "B2RError", "heat_3D_gpu_main", "gol_3D_gpu_main", "lib", "LIB_PATH",
           "MODEL_HEAT", "MODEL_GOL", "MODEL_EQWP_REF", "MODEL_EQWP_STAG", "BC_SHELL",
           "BC_PERIODIC", "FIELDS"]

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libb2r.so")

MODEL_HEAT, MODEL_GOL, MODEL_EQWP_REF, MODEL_EQWP_STAG = 1, 2, 3, 4
BC_SHELL, BC_PERIODIC = 0, 1
FIELDS = {"vx": 0, "vy": 1, "vz": 2, "sxx": 3, "sxy": 4, "sxz": 5, "syy": 6, "syz": 7,
          "szz": 8, "disp": 9, "lambda": 16, "mu": 17, "buoy": 18, "kappa": 19}
_STATUS = {0: "B2R_OK", 1: "B2R_ERR_ARG", 2: "B2R_ERR_CUDA", 3: "B2R_ERR_OOM",
           4: "B2R_ERR_TIMEOUT", 5: "B2R_ERR_STATE"}


class B2RError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{_STATUS.get(status, status)}: {msg}")
        self.status = status


class Config(C.Structure):
    _fields_ = [("model", C.c_int), ("env", C.c_int * 3), ("blocks", C.c_int * 3),
                ("R", C.c_int), ("D", C.c_int), ("boundary", C.c_int),
                ("alpha_dt", C.c_double), ("dx", C.c_double), ("dy", C.c_double),
                ("dz", C.c_double), ("dt", C.c_double), ("h", C.c_double),
                ("src", C.c_int * 3)]


class BatchItem(C.Structure):
    _fields_ = [("env", C.c_int * 3), ("D", C.c_int), ("nsteps", C.c_int),
                ("alpha_dt", C.c_double), ("dx", C.c_double), ("dy", C.c_double),
                ("dz", C.c_double)]


_lib = None


def lib():
    """Load libb2r.so (raises if it was not built: there is no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing; run __graft_entry__.build() first")
    L = C.CDLL(LIB_PATH)
    vp, i, d = C.c_void_p, C.c_int, C.c_double
    sig = {
        "b2r_create": ([C.POINTER(Config), C.POINTER(vp)], i),
        "b2r_destroy": ([vp], i),
        "b2r_last_error": ([vp], C.c_char_p),
        "b2r_set_stream": ([vp, vp], i),
        "b2r_synchronize": ([vp], i),
        "b2r_geometry": ([vp, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                          C.POINTER(C.c_int)], i),
        "b2r_cells": ([vp], C.c_int64),
        "b2r_upload": ([vp, i, vp, i], i),
        "b2r_download": ([vp, i, vp, i], i),
        "b2r_download_blocks": ([vp, i, vp, i], i),
        "b2r_step": ([vp, i], i),
        "b2r_set_graphs": ([vp, i], i),
        "b2r_set_tuning": ([vp, i, i], i),
        "b2r_get_tuning": ([vp, i, C.POINTER(i)], i),
        "b2r_autotune": ([vp, i, C.POINTER(C.c_int), C.POINTER(d)], i),
        "b2r_run_host": ([vp, i, vp, i, vp], i),
        "b2r_run_host_batch": ([vp, i, C.POINTER(vp), C.POINTER(vp), i, i], i),
        "b2r_time_step": ([vp], C.c_int64),
        "b2r_set_source": ([vp, C.POINTER(C.c_float), i], i),
        "b2r_boundary_updating_direct": ([vp, i, i], i),
        "b2r_boundary_updating": ([vp, i, i], i),
        "b2r_heat_3D_gpu_main": ([vp, i, i, C.c_char_p, i, i, i, d, d, d, d, vp,
                                  C.POINTER(d)], i),
        "b2r_heat_3D_cpu_main": ([vp, i, i, C.c_char_p, i, i, i, d, d, d, d, i, C.POINTER(d)], i),
        "b2r_heat_3D_hybrid_main": ([vp, i, i, C.c_char_p, i, i, i, d, d, d, d, i, i, vp,
                                     C.POINTER(d)], i),
        "b2r_gol_3D_gpu_main": ([vp, i, C.c_char_p, i, i, i, vp, C.POINTER(d)], i),
        "b2r_eqwp_gpu_main": ([vp, i, i, C.POINTER(d)], i),
        "b2r_write_block_data": ([vp, i, i, i, C.c_char_p, i, C.c_char_p, i], i),
        "b2r_kernel_launches": ([], C.c_int64),
        "b2r_eqwp_record": ([vp, i, i, C.POINTER(C.c_int), C.POINTER(C.c_float)], i),
        "b2r_eqwp_misfit_gradient": ([vp, i, i, C.POINTER(C.c_int), C.POINTER(C.c_float), i,
                                      C.POINTER(d), C.POINTER(d), C.POINTER(d), C.POINTER(d),
                                      C.POINTER(C.c_float)], i),
        "b2r_heat_record": ([vp, i, i, C.POINTER(C.c_int), C.POINTER(C.c_float)], i),
        "b2r_heat_misfit_gradient": ([vp, i, i, C.POINTER(C.c_int), C.POINTER(C.c_float), i,
                                      C.POINTER(d), C.POINTER(d), C.POINTER(C.c_float)], i),
        "b2r_selfcheck_bounded_wait": ([C.c_double, vp], i),
        "b2r_batch_create": ([C.POINTER(BatchItem), i, C.POINTER(vp)], i),
        "b2r_batch_destroy": ([vp], i),
        "b2r_batch_last_error": ([], C.c_char_p),
        "b2r_batch_upload": ([vp, i, vp, i, vp], i),
        "b2r_batch_download": ([vp, i, vp, i, vp], i),
        "b2r_batch_run": ([vp, vp, i], i),
        "b2r_batch_synchronize": ([vp, vp], i),
        "b2r_batch_lups": ([vp], C.c_int64),
        "b2r_batch_set_zchunk": ([vp, i], i),
        "b2r_batch_autotune": ([vp, vp, C.POINTER(C.c_int), C.POINTER(d)], i),
        "b2r_batch_set_tile": ([vp, i], i),
        "b2r_batch_tile": ([vp], i),
        "b2r_batch_instance_tile": ([vp, i], i),
        "b2r_batch_set_pass_steps": ([vp, i], i),
        "b2r_eqwp_batch_create": ([C.POINTER(vp), C.POINTER(i), i, C.POINTER(vp)], i),
        "b2r_eqwp_batch_destroy": ([vp], i),
        "b2r_eqwp_batch_last_error": ([], C.c_char_p),
        "b2r_eqwp_batch_run": ([vp, vp, i], i),
        "b2r_eqwp_batch_synchronize": ([vp, vp], i),
        "b2r_eqwp_batch_lups": ([vp], C.c_int64),
        "b2r_eqwp_batch_set_zchunk": ([vp, i], i),
        "b2r_batch_instance_pass_steps": ([vp, i], i),
    }
    for name, (args, res) in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    _lib = L
    return L


def read_block_data_bin(path):
    """(nz, ny, nx) float32 array of a file in the reference's block data
    format: int32[3] {Ngx, Ngy, Ngz}, then Ngx*Ngy*Ngz floats, x fastest."""
    raw = open(path, "rb").read()
    nx, ny, nz = np.frombuffer(raw[:12], np.int32)
    cells = np.frombuffer(raw[12:], np.float32)
    if cells.size != int(nx) * int(ny) * int(nz):
        raise ValueError("%s: header %dx%dx%d does not match %d cells" % (path, nx, ny, nz, cells.size))
    return cells.reshape(int(nz), int(ny), int(nx))


def _check(st, handle=None):
    if st != 0:
        msg = lib().b2r_last_error(handle)
        raise B2RError(st, msg.decode() if msg else "")


def _ptr(a, need=None, itemsize=None):
    """(pointer, is_device) of a C-contiguous numpy array or torch tensor.

    need: the bytes the library reads or writes through the pointer; an
    array of another size, element size or layout raises ValueError before
    any copy (the library trusts the pointer for that many bytes)."""
    if isinstance(a, np.ndarray):
        contig, nbytes, isz = a.flags.c_contiguous, a.nbytes, a.itemsize
        ptr, dev = a.ctypes.data, 0
    elif hasattr(a, "data_ptr"):
        contig, nbytes, isz = a.is_contiguous(), a.numel() * a.element_size(), a.element_size()
        ptr, dev = a.data_ptr(), 1 if a.is_cuda else 0
    else:
        raise TypeError("expected a numpy array or a torch tensor, got %s" % type(a).__name__)
    if not contig:
        raise ValueError("the array must be C-contiguous")
    if itemsize is not None and isz != itemsize:
        raise ValueError("cells of %d bytes expected, got %d" % (itemsize, isz))
    if need is not None and nbytes != need:
        raise ValueError("the array must hold %d bytes, got %d" % (need, nbytes))
    return C.c_void_p(ptr), dev


def _ef(edge_flag):
    """edge_flag[3] (one of -1, 0, 1 per axis) as the char[3] the library reads."""
    if edge_flag is None:
        return None
    ef = [int(v) for v in edge_flag]
    if len(ef) != 3 or any(v not in (-1, 0, 1) for v in ef):
        raise ValueError("edge_flag holds three values in {-1, 0, 1}, got %r" % (edge_flag,))
    return bytes([(v + 256) % 256 for v in ef])


def _block(h_in, dtype):
    if not isinstance(h_in, np.ndarray) or h_in.dtype != dtype or h_in.ndim != 3 or not h_in.flags.c_contiguous:
        raise ValueError("a C-contiguous 3-D %s numpy block (nz, ny, nx) expected" % np.dtype(dtype).name)
    return h_in.shape


def _traces(d_obs, nsteps, nrec):
    obs = np.ascontiguousarray(d_obs, np.float32)
    if obs.shape != (nsteps, nrec):
        raise ValueError("d_obs must be (nsteps, nrec) = (%d, %d), got %s" % (nsteps, nrec, obs.shape))
    return obs


class Domain:
    """The resident subdomains of one B2R simulation (one b2r handle)."""

    def __init__(self, model, env, blocks=(1, 1, 1), R=1, D=1, boundary=BC_SHELL,
                 alpha_dt=0.01, dx=1.0, dy=1.0, dz=1.0, dt=0.0, h=1.0, src=(0, 0, 0),
                 stream=None):
        cfg = Config()
        cfg.model = model
        cfg.env[:] = list(env)
        cfg.blocks[:] = list(blocks)
        cfg.R, cfg.D, cfg.boundary = R, D, boundary
        cfg.alpha_dt, cfg.dx, cfg.dy, cfg.dz = alpha_dt, dx, dy, dz
        cfg.dt, cfg.h = dt, h
        cfg.src[:] = list(src)
        self.cfg = cfg
        hnd = C.c_void_p()
        _check(lib().b2r_create(C.byref(cfg), C.byref(hnd)))
        self.h = hnd
        if stream is not None:
            self.set_stream(stream)
        bn, dn = (C.c_int * 3)(), (C.c_int * 3)()
        halo, cb = C.c_int(), C.c_int()
        _check(lib().b2r_geometry(self.h, bn, C.byref(halo), dn, C.byref(cb)), self.h)
        self.block_n = tuple(bn)
        self.halo = halo.value
        self.domain_n = tuple(dn)          # x, y, z
        self.cell_bytes = cb.value
        self.dtype = np.uint8 if cb.value == 1 else np.float32

    @property
    def domain_shape(self):
        """numpy shape (nz, ny, nx) of a domain array."""
        return self.domain_n[::-1]

    @property
    def cells(self):
        return int(lib().b2r_cells(self.h))

    @property
    def time_step(self):
        return int(lib().b2r_time_step(self.h))

    def close(self):
        if getattr(self, "h", None):
            lib().b2r_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_stream(self, stream):
        """stream: an int handle or a torch.cuda.Stream."""
        s = getattr(stream, "cuda_stream", stream)
        _check(lib().b2r_set_stream(self.h, C.c_void_p(int(s))), self.h)

    def set_graphs(self, enable):
        """Replay whole periods from CUDA graphs (needs a non-default stream)."""
        _check(lib().b2r_set_graphs(self.h, 1 if enable else 0), self.h)

    def set_tuning(self, zchunk=None, ctas_per_sm=None, pdl=None, tblock=None, zchunk2=None,
                   eqwp_fused=None, gol_bytes=None, adj_fused=None, gol_push=None, tb16=None,
                   tb_narrow=None, tb_r2=None, eqwp_tma=None, eqwp_overlap=None, gol_rows=None):
        """Launch-schedule knobs (B2R_TUNE_* of b2r.h, keys 1..15); None
        leaves a knob as it is.  Every choice gives the same results."""
        for key, v in ((1, zchunk), (2, ctas_per_sm), (3, pdl), (4, tblock), (5, zchunk2),
                       (6, eqwp_fused), (7, gol_bytes), (8, adj_fused), (9, gol_push), (10, tb16),
                       (11, tb_narrow), (12, tb_r2), (13, eqwp_tma), (14, eqwp_overlap), (15, gol_rows)):
            if v is not None:
                _check(lib().b2r_set_tuning(self.h, key, int(v)), self.h)

    def get_tuning(self):
        """Every knob's current value (by the names set_tuning takes)."""
        out = {}
        for key, name in ((1, "zchunk"), (2, "ctas_per_sm"), (3, "pdl"), (4, "tblock"), (5, "zchunk2"),
                          (6, "eqwp_fused"), (7, "gol_bytes"), (8, "adj_fused"), (9, "gol_push"),
                          (10, "tb16"), (11, "tb_narrow"), (12, "tb_r2"), (13, "eqwp_tma"),
                          (14, "eqwp_overlap"), (15, "gol_rows")):
            v = C.c_int()
            _check(lib().b2r_get_tuning(self.h, key, C.byref(v)), self.h)
            out[name] = v.value
        return out

    def autotune(self, trial_steps=4):
        """Pick the fastest launch schedule / kernel choice for this shape
        (heat, Game of Life, staggered elastic wave); returns (the chosen
        knobs as get_tuning names them, ms per step or -1 when cached)."""
        best = (C.c_int * 3)()
        ms = C.c_double()
        _check(lib().b2r_autotune(self.h, trial_steps, best, C.byref(ms)), self.h)
        return self.get_tuning(), ms.value

    def synchronize(self):
        _check(lib().b2r_synchronize(self.h), self.h)

    @property
    def _domain_bytes(self):
        return int(np.prod(self.domain_shape)) * self.cell_bytes

    def _field_cell_bytes(self, field):
        # material and conductivity fields are float32 whatever the model's cells
        return 4 if FIELDS.get(field, field) >= 16 else self.cell_bytes

    def upload(self, arr, field=0):
        isz = self._field_cell_bytes(field)
        p, dev = _ptr(arr, int(np.prod(self.domain_shape)) * isz, isz)
        _check(lib().b2r_upload(self.h, FIELDS.get(field, field), p, dev), self.h)

    def download(self, out=None, field=0):
        if out is None:
            out = np.empty(self.domain_shape, self.dtype)
        p, dev = _ptr(out, self._domain_bytes, self.cell_bytes)
        _check(lib().b2r_download(self.h, FIELDS.get(field, field), p, dev), self.h)
        return out

    def download_blocks(self, field=0):
        """dict {(bx,by,bz): padded block (nz,ny,nx)} with halos, as stored."""
        nb = tuple(self.cfg.blocks)
        n = self.block_n
        out = np.empty((nb[0] * nb[1] * nb[2], n[2], n[1], n[0]), self.dtype)
        p, dev = _ptr(out)
        _check(lib().b2r_download_blocks(self.h, FIELDS.get(field, field), p, dev), self.h)
        res = {}
        for bz in range(nb[2]):
            for by in range(nb[1]):
                for bx in range(nb[0]):
                    res[(bx, by, bz)] = out[bx + nb[0] * (by + nb[1] * bz)]
        return res

    def write_block_data(self, field=0, block=0, time_step=None, directory=None, text=False):
        """Write one padded block of a field as the reference's
        write_block_data_bin / write_block_data (eqwp.cu:616-651) do: an
        int32[3] {Ngx, Ngy, Ngz} header and the float cells (x fastest), or
        comma-separated text, one line per row.  Returns the path written."""
        ts = self.time_step if time_step is None else int(time_step)
        buf = C.create_string_buffer(4096)
        d = None if directory is None else os.fsencode(directory)
        _check(lib().b2r_write_block_data(self.h, FIELDS.get(field, field), int(block), ts, d,
                                          1 if text else 0, buf, len(buf)), self.h)
        return buf.value.decode()

    def step(self, nsteps):
        _check(lib().b2r_step(self.h, int(nsteps)), self.h)

    def run_host(self, host_in, nsteps, host_out, field=0):
        pi, _ = _ptr(host_in, self._domain_bytes, self.cell_bytes)
        po, _ = _ptr(host_out, self._domain_bytes, self.cell_bytes)
        _check(lib().b2r_run_host(self.h, FIELDS.get(field, field), pi, int(nsteps), po), self.h)
        return host_out

    @property
    def nfields(self):
        """Fields of one problem: the wavefield components of the elastic
        wave (ten with the displacement for the reference model), else one."""
        return {MODEL_EQWP_REF: 10, MODEL_EQWP_STAG: 9}.get(self.cfg.model, 1)

    def run_host_batch(self, host_ins, nsteps, host_outs, field=0):
        """run_host over several independent inputs, the copies of the next
        input and the previous result overlapping the stepping.  Each input
        and output holds the model's `nfields` domain arrays back to back
        (shape (nfields, nz, ny, nx) for the elastic wave)."""
        if len(host_ins) != len(host_outs):
            raise ValueError("one output per input")
        n = len(host_ins)
        need = self._domain_bytes * self.nfields
        pi = (C.c_void_p * max(n, 1))(*[_ptr(a, need, self.cell_bytes)[0].value for a in host_ins])
        po = (C.c_void_p * max(n, 1))(*[_ptr(a, need, self.cell_bytes)[0].value for a in host_outs])
        _check(lib().b2r_run_host_batch(self.h, FIELDS.get(field, field), pi, po, n, int(nsteps)), self.h)
        return host_outs

    def set_source(self, amps):
        a = np.ascontiguousarray(amps, np.float32)
        _check(lib().b2r_set_source(self.h, a.ctypes.data_as(C.POINTER(C.c_float)), a.size),
               self.h)

    def boundary_updating(self, time_step=0, field=0):
        _check(lib().b2r_boundary_updating(self.h, time_step, FIELDS.get(field, field)), self.h)

    def boundary_updating_direct(self, time_step=0, field=0):
        _check(lib().b2r_boundary_updating_direct(self.h, time_step, FIELDS.get(field, field)),
               self.h)

    def eqwp_record(self, nsteps, rec_xyz):
        """vy at receivers (global interior x, y, z) after every step: (nsteps, nrec)."""
        rec = np.ascontiguousarray(rec_xyz, np.int32).reshape(-1, 3)
        out = np.empty((nsteps, len(rec)), np.float32)
        _check(lib().b2r_eqwp_record(self.h, nsteps, len(rec), rec.ctypes.data_as(C.POINTER(C.c_int)),
                                     out.ctypes.data_as(C.POINTER(C.c_float))), self.h)
        return out

    def heat_record(self, nsteps, rec_xyz):
        """u at receivers (global interior x, y, z) after every step of the
        conductivity-scaled heat scheme: (nsteps, nrec)."""
        rec = np.ascontiguousarray(rec_xyz, np.int32).reshape(-1, 3)
        out = np.empty((nsteps, len(rec)), np.float32)
        _check(lib().b2r_heat_record(self.h, nsteps, len(rec), rec.ctypes.data_as(C.POINTER(C.c_int)),
                                     out.ctypes.data_as(C.POINTER(C.c_float))), self.h)
        return out

    def heat_misfit_gradient(self, nsteps, rec_xyz, d_obs, ckpt_every=50):
        """(J, g_kappa, d_syn): the gradient is an env-shaped FP64 array (z, y, x)."""
        rec = np.ascontiguousarray(rec_xyz, np.int32).reshape(-1, 3)
        obs = _traces(d_obs, nsteps, len(rec))
        g = np.empty(tuple(self.cfg.env)[::-1], np.float64)
        J = C.c_double()
        syn = np.empty((nsteps, len(rec)), np.float32)
        dp = C.POINTER(C.c_double)
        _check(lib().b2r_heat_misfit_gradient(
            self.h, nsteps, len(rec), rec.ctypes.data_as(C.POINTER(C.c_int)),
            obs.ctypes.data_as(C.POINTER(C.c_float)), ckpt_every, C.byref(J), g.ctypes.data_as(dp),
            syn.ctypes.data_as(C.POINTER(C.c_float))), self.h)
        return J.value, g, syn

    def eqwp_misfit_gradient(self, nsteps, rec_xyz, d_obs, ckpt_every=50):
        """(J, (g_lambda, g_mu, g_rho), d_syn): gradients are env-shaped FP64 arrays (z, y, x)."""
        rec = np.ascontiguousarray(rec_xyz, np.int32).reshape(-1, 3)
        obs = _traces(d_obs, nsteps, len(rec))
        env = tuple(self.cfg.env)[::-1]
        g = [np.empty(env, np.float64) for _ in range(3)]
        J = C.c_double()
        syn = np.empty((nsteps, len(rec)), np.float32)
        dp = C.POINTER(C.c_double)
        _check(lib().b2r_eqwp_misfit_gradient(
            self.h, nsteps, len(rec), rec.ctypes.data_as(C.POINTER(C.c_int)),
            obs.ctypes.data_as(C.POINTER(C.c_float)), ckpt_every, C.byref(J),
            g[0].ctypes.data_as(dp), g[1].ctypes.data_as(dp), g[2].ctypes.data_as(dp),
            syn.ctypes.data_as(C.POINTER(C.c_float))), self.h)
        return J.value, tuple(g), syn

    def eqwp_gpu_main(self, ts, R):
        secs = C.c_double()
        _check(lib().b2r_eqwp_gpu_main(self.h, ts, R, C.byref(secs)), self.h)
        return secs.value


def _bcheck(st):
    if st != 0:
        msg = lib().b2r_batch_last_error()
        raise B2RError(st, msg.decode() if msg else "")


def _ebcheck(st):
    if st != 0:
        msg = lib().b2r_eqwp_batch_last_error()
        raise B2RError(st, msg.decode() if msg else "")


class EqwpBatch:
    """Staggered elastic-wave Domains (one block each, fixed shell) advanced
    in one persistent launch (b2r_eqwp_batch_*): each run advances domain i
    by nsteps[i] steps, in place, in stream order with the domains' own
    work.  The domains must outlive the batch."""

    def __init__(self, domains, nsteps, stream=None):
        self.domains = list(domains)
        n = len(self.domains)
        hs = (C.c_void_p * n)(*[d.h.value for d in self.domains])
        ns = (C.c_int * n)(*[int(v) for v in nsteps])
        self.nsteps = [int(v) for v in nsteps]
        hnd = C.c_void_p()
        _ebcheck(lib().b2r_eqwp_batch_create(hs, ns, n, C.byref(hnd)))
        self.h = hnd
        self.stream = C.c_void_p(int(getattr(stream, "cuda_stream", stream) or 0))

    @property
    def lups(self):
        return int(lib().b2r_eqwp_batch_lups(self.h))

    def set_zchunk(self, z):
        _ebcheck(lib().b2r_eqwp_batch_set_zchunk(self.h, int(z)))

    def run(self, graph=True):
        _ebcheck(lib().b2r_eqwp_batch_run(self.h, self.stream, 1 if graph else 0))

    def synchronize(self):
        _ebcheck(lib().b2r_eqwp_batch_synchronize(self.h, self.stream))

    def close(self):
        if getattr(self, "h", None):
            lib().b2r_eqwp_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class Batch:
    """Independent heat instances advanced in one persistent launch (b2r_batch_*).

    items: iterable of dicts with env (x, y, z), D, nsteps and optionally
    alpha_dt, dx, dy, dz.  Instance arrays have a fixed shell of D cells."""

    def __init__(self, items, stream=None):
        items = list(items)
        arr = (BatchItem * len(items))()
        for k, it in enumerate(items):
            arr[k].env[:] = list(it["env"])
            arr[k].D = it["D"]
            arr[k].nsteps = it["nsteps"]
            arr[k].alpha_dt = it.get("alpha_dt", 0.01)
            arr[k].dx, arr[k].dy, arr[k].dz = it.get("dx", 1.0), it.get("dy", 1.0), it.get("dz", 1.0)
        self.items = items
        hnd = C.c_void_p()
        _bcheck(lib().b2r_batch_create(arr, len(items), C.byref(hnd)))
        self.h = hnd
        self.stream = C.c_void_p(int(getattr(stream, "cuda_stream", stream) or 0))

    def shape(self, i):
        it = self.items[i]
        return tuple(e + 2 * it["D"] for e in it["env"][::-1])

    @property
    def lups(self):
        return int(lib().b2r_batch_lups(self.h))

    def _bytes(self, i):
        if not 0 <= i < len(self.items):
            raise IndexError("instance %d of %d" % (i, len(self.items)))
        return int(np.prod(self.shape(i))) * 4

    def upload(self, i, arr):
        p, dev = _ptr(arr, self._bytes(i), 4)
        _bcheck(lib().b2r_batch_upload(self.h, i, p, dev, self.stream))

    def download(self, i, out=None):
        if out is None:
            out = np.empty(self.shape(i), np.float32)
        p, dev = _ptr(out, self._bytes(i), 4)
        _bcheck(lib().b2r_batch_download(self.h, i, p, dev, self.stream))
        return out

    def run(self, graph=True):
        _bcheck(lib().b2r_batch_run(self.h, self.stream, 1 if graph else 0))

    def synchronize(self):
        _bcheck(lib().b2r_batch_synchronize(self.h, self.stream))

    def set_zchunk(self, z):
        _bcheck(lib().b2r_batch_set_zchunk(self.h, int(z)))

    def set_tile(self, width):
        """Tile width of every instance: 128, 64, 32, or 0 for each
        instance's fewest-cells shape (the default)."""
        _bcheck(lib().b2r_batch_set_tile(self.h, int(width)))

    @property
    def tile(self):
        """Tile width shared by every instance, 0 if they differ."""
        return int(lib().b2r_batch_tile(self.h))

    def instance_tiles(self):
        """Tile width of each instance (caller order)."""
        return [int(lib().b2r_batch_instance_tile(self.h, i)) for i in range(len(self.items))]

    def set_pass_steps(self, steps):
        """Time steps per HBM pass of the radius-1 instances: 1 or 2."""
        _bcheck(lib().b2r_batch_set_pass_steps(self.h, int(steps)))

    def instance_pass_steps(self):
        """Time steps per HBM pass of each instance (caller order)."""
        return [int(lib().b2r_batch_instance_pass_steps(self.h, i)) for i in range(len(self.items))]

    def autotune(self):
        z = C.c_int()
        ms = C.c_double()
        _bcheck(lib().b2r_batch_autotune(self.h, self.stream, C.byref(z), C.byref(ms)))
        return z.value, ms.value

    def close(self):
        if getattr(self, "h", None):
            lib().b2r_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def kernel_launches():
    """Kernels launched by libb2r in this process so far."""
    return int(lib().b2r_kernel_launches())


def heat_3D_gpu_main(h_in, R, D=1, edge_flag=None, alpha_dt=0.1 * 0.1, dx=1.0, dy=1.0, dz=0.5,
                     stream=None):
    """heat-3D.cu:583 on a host float32 block (nz,ny,nx), in place; returns GPU seconds."""
    nz, ny, nx = _block(h_in, np.float32)
    secs = C.c_double()
    s = getattr(stream, "cuda_stream", stream) or 0
    _check(lib().b2r_heat_3D_gpu_main(h_in.ctypes.data_as(C.c_void_p), R, D, _ef(edge_flag), nx,
                                      ny, nz, alpha_dt, dx, dy, dz, C.c_void_p(int(s)),
                                      C.byref(secs)))
    return secs.value


def heat_3D_cpu_main(h_in, R, D=1, edge_flag=None, alpha_dt=0.1 * 0.1, dx=1.0, dy=1.0, dz=0.5,
                     nthreads=0):
    """heat-3D.cpp:136 on the host cores, in place on a host float32 block
    (nz,ny,nx), bit-identical to heat_3D_gpu_main; returns wall seconds."""
    nz, ny, nx = _block(h_in, np.float32)
    secs = C.c_double()
    _check(lib().b2r_heat_3D_cpu_main(h_in.ctypes.data_as(C.c_void_p), R, D, _ef(edge_flag), nx, ny, nz,
                                      alpha_dt, dx, dy, dz, int(nthreads), C.byref(secs)))
    return secs.value


def heat_3D_hybrid_main(h_in, R, cpu_planes, D=1, edge_flag=None, alpha_dt=0.1 * 0.1, dx=1.0, dy=1.0,
                        dz=0.5, nthreads=0, stream=None):
    """One block split along z between the host cores (the last cpu_planes
    result planes) and the GPU (the rest), in place, bit-identical to
    heat_3D_gpu_main; returns wall seconds."""
    nz, ny, nx = _block(h_in, np.float32)
    secs = C.c_double()
    s = getattr(stream, "cuda_stream", stream) or 0
    _check(lib().b2r_heat_3D_hybrid_main(h_in.ctypes.data_as(C.c_void_p), R, D, _ef(edge_flag), nx, ny, nz,
                                         alpha_dt, dx, dy, dz, int(cpu_planes), int(nthreads),
                                         C.c_void_p(int(s)), C.byref(secs)))
    return secs.value


def gol_3D_gpu_main(h_in, R, edge_flag=None, stream=None):
    """gol-3D.cu:119 on a host uint8 block (nz,ny,nx), in place; returns GPU seconds."""
    nz, ny, nx = _block(h_in, np.uint8)
    secs = C.c_double()
    s = getattr(stream, "cuda_stream", stream) or 0
    _check(lib().b2r_gol_3D_gpu_main(h_in.ctypes.data_as(C.c_void_p), R, _ef(edge_flag), nx, ny,
                                     nz, C.c_void_p(int(s)), C.byref(secs)))
    return secs.value
