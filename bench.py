"""Benchmark of the B2R stencil hot path on GB300 (GLUPS + HBM roofline).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload heat1_512|heat4_512|heat_128|gol_256|eqwp_stag]

One "step" = one pass of the workload: `sub_steps` time steps over the whole
synthetic domain (e.g. 100 heat steps over 512^3).  Rank 0 prints one JSON
line.  With N > 1 (torchrun) every rank runs an independent replica on its
own GPU (weak scaling, no data-path collective); the timed region is bracketed
by barriers and the slowest rank's time is used.

value      GLUPS over all ranks, inputs resident in HBM (CUDA events on the
           stream the library launches on).
e2e        the same metric through b2r_run_host_batch: pinned host input -> device,
           sub_steps time steps, device -> pinned host output, every step; the
           copies of the next step's input and the previous step's result
           overlap the stepping (two copy streams).  Elastic wave: every step
           uploads and downloads each wavefield component through
           Domain.upload / Domain.download (the material stays resident).
roofline   dominant kernel: algorithmic bytes per launch (bytes_per_cell x
           cells swept by one launch) / average launch time, against the
           measured HBM copy bandwidth.
cpu_baseline  the reference's own heat-3D.cpp (oracle/_ref, where it was
           built) or the oracle's restatement, on this host's cores, over a
           bounded sample of the same workload.
--impl reference  times that CPU implementation alone, one bounded sample
           per step, and prints the same line with "impl": "reference".
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

L2_BYTES = 129 * 2 ** 20

WORKLOADS = {
    # FP32 heat delta1 (fdm_heat_diffuse_delta1), 512^3 interior, fixed zero shell,
    # alpha*dt/dx^2 = 0.1 on every axis, R = 1, one block
    "heat1_512": dict(model=1, env=(512, 512, 512), blocks=(1, 1, 1), R=1, D=1, sub_steps=100,
                      coef=(0.1, 1.0, 1.0, 1.0), bytes_per_cell=8, kernel="heat_sweep_kernel<1>"),
    # the same kernel on 384^3 (226 MB per field, > L2): the profiling case
    "heat1_384": dict(model=1, env=(384, 384, 384), blocks=(1, 1, 1), R=1, D=1, sub_steps=20,
                      coef=(0.1, 1.0, 1.0, 1.0), bytes_per_cell=8, kernel="heat_sweep_kernel<1>"),
    # FP32 heat delta4 (fdm_heat_diffuse_delta4), 512^3
    "heat4_512": dict(model=1, env=(512, 512, 512), blocks=(1, 1, 1), R=1, D=4, sub_steps=100,
                      coef=(0.02, 1.0, 1.0, 1.0), bytes_per_cell=8, kernel="heat_sweep_kernel<4>"),
    # FP32 heat delta2 (fdm_heat_diffuse_delta2), 512^3: the radius-2 temporal-blocking case
    "heat2_512": dict(model=1, env=(512, 512, 512), blocks=(1, 1, 1), R=1, D=2, sub_steps=100,
                      coef=(0.02, 1.0, 1.0, 1.0), bytes_per_cell=8, kernel="heat_sweep_kernel<2>"),
    # heat delta1 on the 128^3 case with the reference's constants (fits in L2)
    "heat_128": dict(model=1, env=(128, 128, 128), blocks=(1, 1, 1), R=1, D=1, sub_steps=100,
                     coef=(0.01, 1.0, 1.0, 0.5), bytes_per_cell=8, kernel="heat_sweep_kernel<1>"),
    # 3-D Game of Life, 256^3 torus, 2x2x2 subdomains, R = 4, 400 generations
    "gol_256": dict(model=2, env=(256, 256, 256), blocks=(2, 2, 2), R=4, D=1, sub_steps=400,
                    bytes_per_cell=2, kernel="gol_bits_period_kernel", periodic=True),
    # 64 independent heat instances, edges U{32,48,..,192} per axis, D U{1..4},
    # steps U[50,500], seed 4, in one persistent launch replayed from a CUDA graph
    "batch64": dict(model=5, n=64, seed=4, env=(0, 0, 0), blocks=(1, 1, 1), R=1, D=0, sub_steps=0,
                    bytes_per_cell=8, kernel="batch_kernel"),
    # 16 independent staggered elastic-wave instances (one block each, fixed shell),
    # edges U{32,48,..,128} per axis, steps U[50,150], seed 6, layered model and a
    # Ricker source at each centre, in one persistent launch replayed from a CUDA graph
    "eqwp_batch16": dict(model=7, n=16, seed=6, env=(0, 0, 0), blocks=(1, 1, 1), R=1, D=2, sub_steps=0,
                         bytes_per_cell=84, kernel="eqwp_batch_kernel"),
    # adjoint gradient of a receiver misfit wrt lambda, mu, rho: 256^3, layered model
    # + 5% Gaussian anomaly (sigma 8 cells) for the observed data, 64 receivers on the
    # top plane, Ricker 12 Hz, 2000 steps, checkpoints every 50 steps
    "adjoint256": dict(model=6, env=(256, 256, 256), blocks=(1, 1, 1), R=1, D=2, sub_steps=2000,
                       nrec=64, ckpt=50, f0=12.0, bytes_per_cell=84, kernel="adjoint"),
    # the reference's collocated elastic-wave model, 512x512x256, one block, R = 1
    "eqwp_ref": dict(model=3, env=(512, 512, 256), blocks=(1, 1, 1), R=1, D=2, sub_steps=100,
                     bytes_per_cell=80, kernel="eqwp_ref_stress+velocity"),
    # staggered elastic wave 512x512x256, 2x2x1 subdomains, R = 2, 100 steps per pass
    "eqwp_stag": dict(model=4, env=(512, 512, 256), blocks=(2, 2, 1), R=2, D=2, sub_steps=100,
                      bytes_per_cell=84, kernel="eqwp_stag_velocity+stress"),
    # the staggered stage kernels on one 256^3 block (1.4 GB on the device): the
    # profiling case of the elastic-wave kernels
    "eqwp_stag_256": dict(model=4, env=(256, 256, 256), blocks=(1, 1, 1), R=1, D=2, sub_steps=20,
                          bytes_per_cell=84, kernel="eqwp_stag_velocity+stress"),
    # the adjoint workload cut to 200 steps (4 checkpoint segments): the
    # profiling case of the reverse sweep
    "adjoint256_200": dict(model=6, env=(256, 256, 256), blocks=(1, 1, 1), R=1, D=2, sub_steps=200,
                           nrec=64, ckpt=50, f0=12.0, bytes_per_cell=84, kernel="adjoint"),
}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="heat1_512", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--tune", default="",
                    help="launch-schedule knobs for Domain.set_tuning, e.g. eqwp_fused=1,tblock=4")
    ap.add_argument("--no-secondary", dest="secondary", action="store_false",
                    help="the default heat1_512 run on one GPU also measures the other configurations "
                         "(under \"secondary\"); this flag skips them")
    return ap.parse_args()


def tuning_of(args):
    kw = {}
    for item in filter(None, args.tune.split(",")):
        k, v = item.split("=")
        kw[k.strip()] = int(v)
    return kw


# ------------------------------------------------------------------ helpers
def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        try:
            return float(json.load(open(p))["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.rows = []
        self.proc = None
        self.idx = str(gpu_index)

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-i", self.idx, "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        if not self.rows:
            return None
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4) if "Active" in r[5 + k]
                          and "Not" not in r[5 + k]})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.rows)}


def seeded_domain(wl, shape, seed=1):
    rng = np.random.default_rng(seed)
    if wl["model"] == 2:
        return (rng.random(shape, dtype=np.float32) < 0.3).astype(np.uint8)
    dom = np.zeros(shape, np.float32)
    D = wl["D"]
    dom[D:-D, D:-D, D:-D] = rng.random(tuple(s - 2 * D for s in shape), dtype=np.float32)
    return dom


# ------------------------------------------------------------------ CPU side
def cpu_sample(wl, budget_s=10.0, nthreads=0, dom=None):
    """Time the reference CPU path on a bounded sample of the workload.

    Heat: the reference's heat_3D_cpu_main (oracle/_ref) when it was built on
    this host, else the oracle's restatement of it (same loop nest).  GoL:
    the oracle's restatement (the reference has no CPU Game of Life).
    Returns (GLUPS, kind, cores, sample-description)."""
    from oracle import orc
    cores = nthreads or os.cpu_count()
    env = wl["env"]
    if wl["model"] == 1:
        D = wl["D"]
        if dom is None:
            dom = seeded_domain(wl, tuple(e + 2 * D for e in env[::-1]))
        use_ref = orc.ref_lib() is not None and D == 1
        kind = "reference" if use_ref else "port"
        steps, t = 0, 0.0
        while t < budget_s or steps < 1:
            t0 = time.perf_counter()
            if use_ref:
                orc.ref_heat_cpu_main(dom, 1, cores)
            else:
                orc.heat_cpu_main(dom, 1, D, *wl["coef"], nthreads=cores)
            t += time.perf_counter() - t0
            steps += 1
        lups = steps * env[0] * env[1] * env[2]
        what = "heat_3D_cpu_main (reference heat-3D.cpp)" if use_ref else "restated heat_3D_cpu_main"
        return lups / t / 1e9, kind, cores, f"{steps} time step(s) of {what} on the full {env} grid"
    if wl["model"] == 2:
        g = seeded_domain(wl, env[::-1]) if dom is None else dom
        steps, t = 0, 0.0
        while t < budget_s or steps < 1:
            t0 = time.perf_counter()
            orc.gol_run_periodic(g, 1, cores)
            t += time.perf_counter() - t0
            steps += 1
        lups = steps * env[0] * env[1] * env[2]
        return lups / t / 1e9, "port", cores, f"{steps} generation(s) of the restated rule on the {env} torus"
    if wl["model"] == 3:
        # the reference's collocated model (eqwp.cu:60-477) restated, on a
        # 128x128x64 sample with its two-cell shell and body force
        n = (128 + 4, 128 + 4, 64 + 4)
        f = [np.zeros(n[::-1], np.float32) for _ in range(10)]
        force = dict(fy=n[1] - 7 - 2, fx0=n[0] // 2, fx1=n[0] // 2 + n[0] // 10, fz0=n[2] // 2,
                     fz1=n[2] // 2 + n[2] // 10, fval=-1e4, fsteps=50)
        steps, t = 0, 0.0
        while t < budget_s or steps < 1:
            t0 = time.perf_counter()
            orc.eqwp_ref_substep(f, 0, 2, 63, steps, force)
            t += time.perf_counter() - t0
            steps += 1
        return (steps * 128 * 128 * 64 / t / 1e9, "port", cores,
                f"{steps} step(s) of the restated reference model on 128x128x64")
    # elastic wave: restated staggered step on a 128x128x64 sample
    n = (128 + 8, 128 + 8, 64 + 8)
    f = [np.zeros(n[::-1], np.float32) for _ in range(9)]
    m = [np.full(n[::-1], v, np.float32) for v in (8e9, 8e9, 1 / 2300.0)]
    steps, t = 0, 0.0
    while t < budget_s or steps < 1:
        t0 = time.perf_counter()
        orc.eqwp_stag_step(f, m, 1e-4, 10.0, 0, 4, 63, (64, 64, 32), 1.0)
        t += time.perf_counter() - t0
        steps += 1
    return steps * 128 * 128 * 64 / t / 1e9, "port", cores, f"{steps} step(s) of the restated staggered scheme on 128x128x64"


def run_reference(args, wl):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import oracle.build as ob
    ob.build_oracle()
    ob.build_ref()
    env = wl["env"]
    D = wl["D"]
    shape = env[::-1] if wl["model"] == 2 else tuple(e + 2 * D for e in env[::-1])
    dom = seeded_domain(wl, shape) if wl["model"] in (1, 2) else None
    # heat / GoL: one full-grid step per bench step; elastic wave: about a
    # second of steps on its sample, so that the arrays' first touch does
    # not dominate
    budget = 1.0 if wl["model"] in (3, 4) else 0.0
    for _ in range(args.warmup):
        cpu_sample(wl, budget_s=budget, dom=dom)
    vals, kind, cores, sample = [], None, None, None
    t_all = 0.0
    for _ in range(args.steps):
        t0 = time.perf_counter()
        v, kind, cores, sample = cpu_sample(wl, budget_s=budget, dom=dom)
        t_all += time.perf_counter() - t0
        vals.append(v)
    value = float(np.mean(vals))
    # for context: the reference's own GPU kernel of the same path
    # (fdm_heat_diffuse_delta1, compiled unmodified), device-resident
    ref_gpu = None
    if wl["model"] == 1 and D == 1:
        try:
            import torch
            from oracle import refgpu
            if torch.cuda.is_available() and refgpu.heat_available():
                ms = refgpu.time_reference_heat(dom, wl["sub_steps"], reps=max(1, args.steps))
                cells = env[0] * env[1] * env[2]
                ref_gpu = {"value": round(cells * wl["sub_steps"] / (ms / 1e3) / 1e9, 3), "unit": "GLUPS",
                           "kernel": "fdm_heat_diffuse_delta1 (heat-3D.cu:173), its own constants",
                           "note": "the reference's CUDA kernel on this GPU, fields resident, no copies"}
        except Exception as e:   # context only: never fails the reference line
            ref_gpu = {"unavailable": str(e)[:200]}
    if wl["model"] == 2:
        try:
            import torch
            from oracle import refgpu
            if torch.cuda.is_available() and refgpu.gol_available():
                shape = tuple(e + 2 for e in env[::-1])     # one block with a one-cell shell
                ms = refgpu.time_reference_gol(shape, wl["sub_steps"], reps=1)
                cells = env[0] * env[1] * env[2]
                ref_gpu = {"value": round(cells * wl["sub_steps"] / (ms / 1e3) / 1e9, 3), "unit": "GLUPS",
                           "kernel": "gol_3d_kernel (gol-3D.cu:30)",
                           "note": "the reference's CUDA kernel on this GPU, one block, resident; timing only "
                                   "(beyond one 32x32 tile its results are wrong at tile edges)"}
        except Exception as e:
            ref_gpu = {"unavailable": str(e)[:200]}
    if wl["model"] == 3:
        try:
            import torch
            from oracle import refgpu
            if torch.cuda.is_available() and refgpu.available():
                shape = tuple(e + 4 for e in env[::-1])     # the reference block, R = 1
                ms = refgpu.time_reference_eqwp(shape, wl["sub_steps"], reps=1)
                cells = env[0] * env[1] * env[2]
                ref_gpu = {"value": round(cells * wl["sub_steps"] / (ms / 1e3) / 1e9, 3), "unit": "GLUPS",
                           "kernel": "eqwp_fd4_stress + eqwp_fd4_v{x,y,z} (eqwp.cu:60-477)",
                           "note": "the reference's CUDA kernels on this GPU, fields resident; timing only "
                                   "(beyond one 16-row tile in y their results are wrong at tile edges)"}
        except Exception as e:
            ref_gpu = {"unavailable": str(e)[:200]}
    line = {"metric": "GLUPS", "value": round(value, 4), "unit": "GLUPS", "impl": "reference",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(1000 * t_all / args.steps, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32" if wl["model"] != 2 else "u8",
            "data": "synthetic (seeded)", "config": config_of(args, wl),
            "cpu_baseline": {"value": round(value, 4), "unit": "GLUPS", "cores": cores, "kind": kind,
                             "sample": sample},
            "e2e": {"value": round(value, 4), "unit": "GLUPS", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            **({"reference_gpu_kernel": ref_gpu} if ref_gpu else {})}
    print(json.dumps(line), flush=True)


def config_of(args, wl):
    cells = wl["env"][0] * wl["env"][1] * wl["env"][2]
    foot = cells * (1 if wl["model"] == 2 else 4) * (2 if wl["model"] in (1, 2) else 12)
    return {"workload": args.workload, "env": list(wl["env"]), "blocks": list(wl["blocks"]),
            "R": wl["R"], "D": wl["D"], "time_steps_per_step": wl["sub_steps"],
            "coef": list(wl.get("coef", [])), "periodic": bool(wl.get("periodic", False)),
            "l2": ("inputs larger than L2" if foot > L2_BYTES else "L2 flushed between timed steps"),
            "parallelism": f"replicas x{args.gpus}", **({"tuning": tuning_of(args)} if args.tune else {})}


# ------------------------------------------------------------------ ranks
def max_over_ranks(ms, dev, world):
    """The slowest rank's time (the job ends with it); world == 1: ms."""
    if world <= 1:
        return float(ms)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(ms)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replicas_glups(world, cells, steps, ms):
    """Whole-job throughput of `world` independent replicas, each advancing
    `cells` cells `steps` times, timed by the slowest rank (ms)."""
    return world * cells * steps / (ms / 1000.0) / 1e9


# ------------------------------------------------------------------ GPU side
def make_domain(b2r, wl, stream):
    kw = dict(blocks=wl["blocks"], R=wl["R"], D=wl["D"], stream=stream,
              boundary=b2r.BC_PERIODIC if wl.get("periodic") else b2r.BC_SHELL)
    if wl["model"] == 1:
        a, dx, dy, dz = wl["coef"]
        kw.update(alpha_dt=a, dx=dx, dy=dy, dz=dz)
    if wl["model"] == 4:
        h = 10.0
        kw.update(h=h, dt=0.5 * h / (4000 * 3 ** 0.5 * (9 / 8 + 1 / 24)),
                  src=tuple(e // 2 for e in wl["env"]))
    return b2r.Domain(wl["model"], wl["env"], **kw)


def load_inputs(d, wl, torch, dev):
    """Seeded inputs, created on the host and uploaded once (resident in HBM)."""
    if wl["model"] in (1, 2):
        host = seeded_domain(wl, d.domain_shape)
        d.upload(host)
        return host
    if wl["model"] == 3:
        zero = np.zeros(d.domain_shape, np.float32)
        for k in range(10):
            d.upload(zero, field=k)
        return zero
    mat, amps = stag_model(d.domain_shape, d.cfg.dt, wl["sub_steps"] * 64)
    for name, arr in zip(("lambda", "mu", "buoy"), mat):
        d.upload(arr, field=name)
    zero = np.zeros(d.domain_shape, np.float32)
    for k in range(9):
        d.upload(zero, field=k)
    d.set_source(amps)
    return zero


def stag_model(shape, dt, nsrc):
    """The staggered elastic-wave workload's material and source: 8 horizontal
    layers (along y) with vp U[2000, 4000] m/s, vs = vp / sqrt(3), rho
    U[2000, 2600] kg/m^3 from seed 3, on a domain array of numpy shape
    (nz, ny, nx); the explosive Ricker source (10 Hz, delayed 1.2 / f0) for
    nsrc steps of dt.  Returns ([lambda, mu, 1/rho] float32, amps float32)."""
    rng = np.random.default_rng(3)
    layers = 8
    vp_l = rng.uniform(2000, 4000, layers)
    rho_l = rng.uniform(2000, 2600, layers)
    idx = np.minimum(np.arange(shape[1]) * layers // shape[1], layers - 1)
    vp = np.broadcast_to(vp_l[idx][None, :, None], shape)
    rho = np.broadcast_to(rho_l[idx][None, :, None], shape)
    mu = rho * (vp / 3 ** 0.5) ** 2
    lam = rho * vp ** 2 - 2 * mu
    mat = [np.ascontiguousarray(arr, np.float32) for arr in (lam, mu, 1.0 / rho)]
    t = np.arange(nsrc) * dt - 1.2 / 10.0
    a = (np.pi * 10.0 * t) ** 2
    return mat, (1e6 * dt * (1 - 2 * a) * np.exp(-a)).astype(np.float32)


def batch_items(wl):
    rng = np.random.default_rng(wl["seed"])
    edges = np.arange(32, 193, 16)
    items = []
    for _ in range(wl["n"]):
        items.append(dict(env=tuple(int(v) for v in rng.choice(edges, 3)), D=int(rng.integers(1, 5)),
                          nsteps=int(rng.integers(50, 501)), alpha_dt=0.02, dx=1.0, dy=1.0, dz=1.0))
    return items


def run_batch(args, wl):
    """Config 4: batched instances vs the same instances as sequential plain runs."""
    import torch
    import __graft_entry__
    __graft_entry__.build()
    import b2r_gb300 as b2r
    dev = torch.device("cuda", 0)
    items = batch_items(wl)
    rng = np.random.default_rng(wl["seed"] + 1)
    ins = []
    for it in items:
        D = it["D"]
        a = np.zeros(tuple(e + 2 * D for e in it["env"][::-1]), np.float32)
        a[D:-D, D:-D, D:-D] = rng.random(it["env"][::-1], dtype=np.float32)
        ins.append(a)
    stream = torch.cuda.Stream(device=dev)
    bt = b2r.Batch(items, stream=stream)
    for i, a in enumerate(ins):
        bt.upload(i, a)
    tuned = bt.autotune()
    widths = bt.instance_tiles()
    # instances per tile width and on two-step units, as the autotuner left
    # them (per order and size class)
    tuned_tile = {str(w): widths.count(w) for w in (128, 64, 32) if w in widths}
    tuned_tile["two_step"] = bt.instance_pass_steps().count(2)
    lups = bt.lups
    for _ in range(args.warmup):
        bt.run()
    bt.synchronize()
    clocks = ClockSampler(0)
    clocks.start()
    l0 = b2r.kernel_launches()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        bt.run()
    e1.record(stream)
    e1.synchronize()
    launches = b2r.kernel_launches() - l0
    bt.synchronize()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1) / args.steps
    value = lups / (ms / 1e3) / 1e9
    # one more run from the inputs for the comparison (the timed runs restart
    # from whatever the previous run left in the buffers)
    for i, a in enumerate(ins):
        bt.upload(i, a)
    bt.run()
    bt.synchronize()
    got = [bt.download(i) for i in range(len(items))]
    # the same instances as sequential plain runs (one handle each, graphs on)
    seq_ms = 0.0
    max_rel = 0.0
    for i, it in enumerate(items):
        with b2r.Domain(b2r.MODEL_HEAT, it["env"], D=it["D"], alpha_dt=0.02, stream=stream) as d:
            d.upload(ins[i])
            d.step(it["nsteps"])              # warm the graphs
            d.upload(ins[i])
            d.synchronize()
            a0 = torch.cuda.Event(enable_timing=True)
            a1 = torch.cuda.Event(enable_timing=True)
            a0.record(stream)
            d.step(it["nsteps"])
            a1.record(stream)
            a1.synchronize()
            seq_ms += a0.elapsed_time(a1)
            plain = d.download()
        max_rel = max(max_rel, float(np.linalg.norm(got[i].astype(np.float64) - plain) /
                                     np.linalg.norm(plain.astype(np.float64))))
    seq = lups / (seq_ms / 1e3) / 1e9
    # the three instances with the fewest updates against the oracle (FP32, FP64)
    from oracle import orc
    small = sorted(range(len(items)), key=lambda i: int(np.prod(items[i]["env"])) * items[i]["nsteps"])[:3]
    r32, r64 = 0.0, 0.0
    for i in small:
        it = items[i]
        a32 = ins[i].copy()
        orc.heat_run(a32, it["D"], it["D"], it["nsteps"], it["alpha_dt"], it["dx"], it["dy"], it["dz"])
        a64 = ins[i].astype(np.float64)
        orc.heat_run(a64, it["D"], it["D"], it["nsteps"], it["alpha_dt"], it["dx"], it["dy"], it["dz"])
        r32, r64 = max(r32, rel_l2(got[i], a32)), max(r64, rel_l2(got[i], a64))
    parity = {"instances": [dict(env=list(items[i]["env"]), D=items[i]["D"], nsteps=items[i]["nsteps"])
                            for i in small],
              "rel_l2_fp32": r32, "rel_l2_fp64": r64, "tolerance": 1e-5,
              "max_rel_l2_vs_sequential": max_rel,
              "oracle": "oracle/b2r_oracle.c heat restatement (FP32, FP64), worst of the three"}
    peak, peak_src = measured_peak()
    achieved = wl["bytes_per_cell"] * lups / (ms / 1e3) / 1e9
    bt.close()
    line = {"metric": "GLUPS", "value": round(value, 3), "unit": "GLUPS", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded U[0,1))",
            "config": {"workload": args.workload, "instances": len(items), "lups_per_step": lups,
                       "autotuned_zchunk": tuned[0], "autotuned_tile_widths": tuned_tile,
                       "sequential_plain_glups": round(seq, 3),
                       "batched_over_sequential": round(value / seq, 3),
                       "max_rel_l2_vs_sequential": max_rel,
                       "l2": "inputs larger than L2"},
            "e2e": None, "gpu_launches": int(launches),
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4), "traffic": None, "peak_source": peak_src,
                         "kernel": "batch_kernel", "note": "8 B per lattice-site update, whole run"},
            "cpu_baseline": None, "clocks": clk, "parity": parity}
    return line


def eqwp_batch_items(wl):
    rng = np.random.default_rng(wl["seed"])
    edges = np.arange(32, 129, 16)
    return [dict(env=tuple(int(v) for v in rng.choice(edges, 3)), nsteps=int(rng.integers(50, 151)))
            for _ in range(wl["n"])]


def run_eqwp_batch(args, wl):
    """Batched staggered elastic-wave instances vs the same handles stepped
    one after the other (two-pass step, graphs of their own)."""
    import torch
    import __graft_entry__
    __graft_entry__.build()
    import b2r_gb300 as b2r
    items = eqwp_batch_items(wl)
    stream = torch.cuda.Stream(device=torch.device("cuda", 0))
    h = 10.0
    dt = 0.5 * h / (4000 * 3 ** 0.5 * (9 / 8 + 1 / 24))

    def domains(st):
        out = []
        for it in items:
            d = b2r.Domain(4, it["env"], D=2, R=1, dt=dt, h=h, src=tuple(e // 2 for e in it["env"]), stream=st)
            mat, amps = stag_model(d.domain_shape, dt, 64 * max(i["nsteps"] for i in items))
            for name, arr in zip(("lambda", "mu", "buoy"), mat):
                d.upload(arr, field=name)
            zero = np.zeros(d.domain_shape, np.float32)
            for k in range(9):
                d.upload(zero, field=k)
            d.set_source(amps)
            d.synchronize()
            out.append(d)
        return out

    doms = domains(stream)
    bt = b2r.EqwpBatch(doms, [it["nsteps"] for it in items], stream=stream)
    lups = bt.lups
    for _ in range(args.warmup):
        bt.run()
    bt.synchronize()
    clocks = ClockSampler(0)
    clocks.start()
    l0 = b2r.kernel_launches()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        bt.run()
    e1.record(stream)
    e1.synchronize()
    launches = b2r.kernel_launches() - l0
    bt.synchronize()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1) / args.steps
    value = lups / (ms / 1e3) / 1e9
    # the same handles, state and time steps included, stepped one after the
    # other: timed, then compared field by field with the batch's next run
    refs = domains(stream)
    runs = args.warmup + args.steps
    for r, it in zip(refs, items):
        r.step(runs * it["nsteps"])
    for r in refs:
        r.synchronize()
    seq_ms = 0.0
    for r, it in zip(refs, items):
        a0 = torch.cuda.Event(enable_timing=True)
        a1 = torch.cuda.Event(enable_timing=True)
        a0.record(stream)
        r.step(it["nsteps"])
        a1.record(stream)
        a1.synchronize()
        seq_ms += a0.elapsed_time(a1)
    bt.run()
    bt.synchronize()
    identical = all(np.array_equal(d.download(field=k), r.download(field=k))
                    for d, r in zip(doms, refs) for k in range(9))
    seq = lups / (seq_ms / 1e3) / 1e9
    peak, peak_src = measured_peak()
    achieved = wl["bytes_per_cell"] * lups / (ms / 1e3) / 1e9
    bt.close()
    for d in doms + refs:
        d.close()
    return {"metric": "GLUPS", "value": round(value, 3), "unit": "GLUPS", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded layered model, Ricker source)",
            "config": {"workload": args.workload, "instances": len(items), "lups_per_step": lups,
                       "sequential_plain_glups": round(seq, 3), "batched_over_sequential": round(value / seq, 3),
                       "l2": "inputs larger than L2"},
            "e2e": None, "gpu_launches": int(launches),
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4), "traffic": None, "peak_source": peak_src,
                         "kernel": "eqwp_batch_kernel", "note": "84 B per cell-step, whole run"},
            "cpu_baseline": None, "clocks": clk,
            "parity": {"bit_identical_to_handles": identical,
                       "note": "every field of every instance against the same handle stepped alone "
                               "(two-pass step), which the GPU tests hold bit-identical to the FP32 oracle"}}


def run_adjoint(args, wl):
    """Config 5: misfit gradient by the adjoint vs one forward of the same run."""
    import torch
    import __graft_entry__
    __graft_entry__.build()
    import b2r_gb300 as b2r
    env, n = wl["env"], wl["sub_steps"]
    h = 10.0
    dt = 0.5 * h / (4400 * 3 ** 0.5 * (9 / 8 + 1 / 24))
    src = tuple(e // 2 for e in env)
    rng = np.random.default_rng(3)
    layers = 8
    vp_l = rng.uniform(2000, 4000, layers)
    rho_l = rng.uniform(2000, 2600, layers)
    shape = tuple(e + 4 for e in env[::-1])
    idx = np.minimum(np.arange(shape[1]) * layers // shape[1], layers - 1)

    def model(anomaly):
        vp = np.broadcast_to(vp_l[idx][None, :, None], shape).astype(np.float64)
        rho = np.broadcast_to(rho_l[idx][None, :, None], shape).astype(np.float64)
        if anomaly:
            z = np.arange(shape[0])[:, None, None] - shape[0] / 2
            y = np.arange(shape[1])[None, :, None] - shape[1] / 2
            x = np.arange(shape[2])[None, None, :] - shape[2] / 2
            vp = vp * (1 + anomaly * np.exp(-(x * x + y * y + z * z) / (2 * 8.0 ** 2)))
        mu = rho * (vp / 3 ** 0.5) ** 2
        return [rho * vp ** 2 - 2 * mu, mu, 1.0 / rho]

    t = np.arange(n) * dt - 1.2 / wl["f0"]
    a = (np.pi * wl["f0"] * t) ** 2
    amps = (1e7 * dt * (1 - 2 * a) * np.exp(-a)).astype(np.float32)
    k = int(np.sqrt(wl["nrec"]))
    gx = np.linspace(8, env[0] - 9, k).astype(np.int32)
    gz = np.linspace(8, env[2] - 9, k).astype(np.int32)
    rec = np.array([(x, 2, z) for x in gx for z in gz], np.int32)

    def domain(mat):
        d = b2r.Domain(b2r.MODEL_EQWP_STAG, env, D=2, R=1, dt=dt, h=h, src=src)
        for name, m in zip(("lambda", "mu", "buoy"), mat):
            d.upload(np.ascontiguousarray(m, np.float32), field=name)
        zero = np.zeros(d.domain_shape, np.float32)
        for f in range(9):
            d.upload(zero, field=f)
        d.set_source(amps)
        return d, zero

    d, zero = domain(model(0.05))
    d_obs = d.eqwp_record(n, rec)
    d.close()
    d, zero = domain(model(0.0))
    tune = tuning_of(args)
    if tune:
        d.set_tuning(**tune)
    torch.cuda.synchronize()
    fwd_ms = []
    for _ in range(max(1, args.warmup // 2)):
        for f in range(9):
            d.upload(zero, field=f)
        t0 = time.perf_counter()
        d.eqwp_record(n, rec)
        fwd_ms.append((time.perf_counter() - t0) * 1e3)
    # one untimed gradient: allocates the workspace the timed calls reuse
    for f in range(9):
        d.upload(zero, field=f)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    d.eqwp_misfit_gradient(n, rec, d_obs, ckpt_every=wl["ckpt"])
    first_ms = (time.perf_counter() - t0) * 1e3
    clocks = ClockSampler(0)
    clocks.start()
    l0 = b2r.kernel_launches()
    grad_ms = []
    for _ in range(max(1, args.steps)):
        for f in range(9):
            d.upload(zero, field=f)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        J, g, _ = d.eqwp_misfit_gradient(n, rec, d_obs, ckpt_every=wl["ckpt"])
        grad_ms.append((time.perf_counter() - t0) * 1e3)
    launches = b2r.kernel_launches() - l0
    clk = clocks.stop()
    for f in range(9):
        d.upload(zero, field=f)
    t0 = time.perf_counter()
    d.eqwp_record(n, rec)
    fwd_ms.append((time.perf_counter() - t0) * 1e3)
    d.close()
    # parity: the gradient's derivative along the anomaly (the model
    # difference that made the observed data) against a central finite
    # difference of the misfit, two more forwards at the full size
    m0, m1 = model(0.0), model(0.05)
    delta = [b - a for a, b in zip(m0, m1)]
    inner = (slice(2, -2),) * 3
    an = float(sum((gk * dk[inner]).sum() for gk, dk in zip(g[:2], delta[:2])))
    eps = 0.05

    def misfit_at(s):
        dd, _ = domain([a + s * eps * dl for a, dl in zip(m0, delta)])
        syn = dd.eqwp_record(n, rec)
        dd.close()
        return 0.5 * float(((syn.astype(np.float64) - d_obs) ** 2).sum())

    fd = (misfit_at(1) - misfit_at(-1)) / (2 * eps)
    parity = {"direction": "the 5 % Gaussian anomaly of vp (lambda, mu)", "adjoint": an,
              "central_difference": fd, "rel_diff": abs(fd - an) / max(abs(fd), 1e-300),
              "eps": eps, "note": "FP64 gradient oracle at 64^3 and 16-direction differences: the GPU tests"}
    cells = env[0] * env[1] * env[2]
    gms = float(np.median(grad_ms))
    fms = float(np.median(fwd_ms))
    value = cells * n / (gms / 1e3) / 1e9
    peak, peak_src = measured_peak()
    line = {"metric": "GLUPS", "value": round(value, 3), "unit": "GLUPS", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(gms, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded layered model, Gaussian anomaly, Ricker source)",
            "config": {"workload": args.workload, "env": list(env), "time_steps": n,
                       "receivers": len(rec), "checkpoint_every": wl["ckpt"],
                       "forward_ms": round(fms, 1), "gradient_ms": round(gms, 1),
                       "first_gradient_ms": round(first_ms, 1),
                       "gradient_over_forward": round(gms / fms, 3),
                       "reverse_over_forward": round((gms - fms) / fms, 3), "misfit": J,
                       "l2": "inputs larger than L2", **({"tuning": tune} if tune else {})},
            "e2e": None, "gpu_launches": int(launches),
            "roofline": {"bound": "hbm", "achieved": round(wl["bytes_per_cell"] * value, 1),
                         "peak": peak, "unit": "GB/s",
                         "frac": round(wl["bytes_per_cell"] * value / peak, 4), "traffic": None,
                         "peak_source": peak_src, "kernel": "adjoint (whole gradient)",
                         "note": "84 B per cell-step of the forward, over the whole gradient time"},
            "cpu_baseline": None, "clocks": clk, "parity": parity}
    return line


def parity_sample(d, wl, host):
    """A short run of the timed schedule (the knobs the handle holds) from the
    workload's own seeded input, checked against the oracle after the timed
    region: heat against the FP32 and FP64 restatements, Game of Life bit for
    bit, the elastic waves against the FP32 and FP64 restatements."""
    from oracle import orc
    model = wl["model"]
    if model == 1:
        D = wl["D"]
        n = 4
        d.upload(host)
        d.step(n)
        got = d.download()
        r32 = host.copy()
        orc.heat_run(r32, D, D, n, *wl["coef"])
        r64 = host.astype(np.float64)
        orc.heat_run(r64, D, D, n, *wl["coef"])
        return {"time_steps": n, "rel_l2_fp32": rel_l2(got, r32), "rel_l2_fp64": rel_l2(got, r64),
                "tolerance": 1e-5, "oracle": "oracle/b2r_oracle.c heat restatement (FP32, FP64)"}
    if model == 2:
        n = 2 * wl["R"]
        d.upload(host)
        d.step(n)
        got = d.download()
        ref = host.copy()
        orc.gol_run_periodic(ref, n)
        bad = int(np.count_nonzero(got != ref))
        return {"generations": n, "bit_exact": bad == 0, "mismatched_cells": bad,
                "oracle": "oracle/b2r_oracle.c rule restatement"}
    if model == 4:
        n = 2 * wl["R"]
        mat, amps = stag_model(d.domain_shape, d.cfg.dt, n)
        rng = np.random.default_rng(12)
        init = []
        for k in range(9):
            f = np.zeros(d.domain_shape, np.float32)
            f[4:-4, 4:-4, 4:-4] = ((rng.random(tuple(v - 8 for v in f.shape), dtype=np.float32) - 0.5) *
                                   (1e-3 if k < 3 else 1e5))
            init.append(f)
            d.upload(f, field=k)
        d.set_source(amps)
        d.step(n)
        got = [d.download(field=k) for k in range(9)]
        src = tuple(int(v) + 2 for v in d.cfg.src)
        f32 = [a.copy() for a in init]
        f64 = [a.astype(np.float64) for a in init]
        m64 = [m.astype(np.float64) for m in mat]
        for t in range(n):
            orc.eqwp_stag_step(f32, mat, d.cfg.dt, d.cfg.h, 0, 2, 63, src, float(amps[t]))
            orc.eqwp_stag_step(f64, m64, d.cfg.dt, d.cfg.h, 0, 2, 63, src, float(amps[t]))
        return {"time_steps": n, "input": "random wavefield, the workload's material and source",
                "bit_identical_fp32": all(np.array_equal(got[k], f32[k]) for k in range(9)),
                "rel_l2_fp32": max(rel_l2(got[k], f32[k]) for k in range(9)),
                "rel_l2_fp64": max(rel_l2(got[k], f64[k]) for k in range(9)), "tolerance": 1e-5,
                "oracle": "oracle/b2r_oracle.c staggered restatement (FP32, FP64), worst of 9 fields"}
    return None


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def run_ours(args, wl):
    import torch
    import torch.distributed as dist
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    import __graft_entry__
    if rank == 0 or world == 1:
        __graft_entry__.build()
    if world > 1:
        dist.barrier()
    import b2r_gb300 as b2r

    def barrier():
        if world > 1:
            dist.barrier()

    stream = torch.cuda.Stream(device=dev)
    d = make_domain(b2r, wl, stream)
    tune = tuning_of(args)
    if tune:
        d.set_tuning(**tune)
    host = load_inputs(d, wl, torch, dev)
    d.synchronize()
    # the library's autotuner picks the launch schedule / kernel choice for
    # this shape (timed on the live fields, which it restores); not part of
    # the timing
    tuned = None
    knobs = {1: ("zchunk", "ctas_per_sm", "pdl", "tblock", "zchunk2", "tb16", "tb_narrow", "tb_r2"),
             2: ("tblock", "gol_bytes", "gol_push", "gol_rows"), 4: ("eqwp_fused", "eqwp_tma", "eqwp_overlap")}
    if wl["model"] in knobs and not tune:
        d.autotune(trial_steps=4)
        tuned = {k: v for k, v in d.get_tuning().items() if k in knobs[wl["model"]]}
    n = wl["sub_steps"]
    cells = wl["env"][0] * wl["env"][1] * wl["env"][2]
    small = config_of(args, wl)["l2"] != "inputs larger than L2"
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device=dev) if small else None

    for _ in range(args.warmup):
        d.step(n)
    d.synchronize()

    # ---- device-resident timed region
    clocks = ClockSampler(local)
    clocks.start()
    barrier()
    torch.cuda.synchronize(dev)
    l0 = b2r.kernel_launches()
    total_ms = 0.0
    if small:
        for _ in range(args.steps):
            with torch.cuda.stream(stream):
                flush.fill_(1.0)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            d.step(n)
            e1.record(stream)
            e1.synchronize()
            total_ms += e0.elapsed_time(e1)
    else:
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            d.step(n)
        e1.record(stream)
        e1.synchronize()
        total_ms = e0.elapsed_time(e1)
    launches = b2r.kernel_launches() - l0
    d.synchronize()
    torch.cuda.synchronize(dev)
    barrier()
    clk = clocks.stop()
    ms = max_over_ranks(total_ms, dev, world) / args.steps
    value = replicas_glups(world, cells, n, ms)

    # ---- e2e through the C ABI with pinned host buffers
    e2e_val, h2d, d2h = None, 0, 0
    if wl["model"] in (1, 2):
        # every step copies its input in and its result out; the copies of
        # step i+1's input and step i-1's result overlap step i's stepping
        pin_in = [torch.from_numpy(host).pin_memory(), torch.from_numpy(host.copy()).pin_memory()]
        pin_out = [torch.empty_like(pin_in[0]).pin_memory() for _ in range(2)]
        d.run_host_batch(pin_in, n, pin_out)        # warm
        barrier()
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        d.run_host_batch([pin_in[k % 2] for k in range(args.steps)], n,
                         [pin_out[k % 2] for k in range(args.steps)])
        torch.cuda.synchronize(dev)
        barrier()
        ems = max_over_ranks((time.perf_counter() - t0) * 1000.0, dev, world) / args.steps
        e2e_val = replicas_glups(world, cells, n, ems)
        h2d = d2h = host.nbytes
    elif wl["model"] in (3, 4):
        # elastic wave: every step uploads the wavefield (its input, every
        # component; the material stays resident) from pinned host memory,
        # runs the time steps and downloads the wavefield; the copies of the
        # next step's wavefield and of the previous result overlap the stepping
        nf = d.nfields
        wave = np.ascontiguousarray(np.broadcast_to(host, (nf,) + host.shape))
        pin_in = [torch.from_numpy(wave).pin_memory(), torch.from_numpy(wave.copy()).pin_memory()]
        pin_out = [torch.empty_like(pin_in[0]).pin_memory() for _ in range(2)]
        d.run_host_batch(pin_in, n, pin_out)        # warm
        barrier()
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        d.run_host_batch([pin_in[k % 2] for k in range(args.steps)], n,
                         [pin_out[k % 2] for k in range(args.steps)])
        torch.cuda.synchronize(dev)
        barrier()
        ems = max_over_ranks((time.perf_counter() - t0) * 1000.0, dev, world) / args.steps
        e2e_val = replicas_glups(world, cells, n, ems)
        h2d = d2h = nf * host.nbytes

    # ---- roofline of the dominant kernel
    peak, peak_src = measured_peak()
    roof = None
    if wl["model"] == 1:
        # algorithmic bytes per launch = 8 B per lattice-site update x the updates
        # one launch performs (cells x time steps per launch: 2 for the radius-1
        # two-step sweep, which reads and writes each cell once per two steps)
        per_launch = launches / args.steps
        steps_per_launch = n / per_launch
        algo = wl["bytes_per_cell"] * cells * steps_per_launch
        per_launch_ms = ms / per_launch
        achieved = algo / (per_launch_ms / 1000.0) / 1e9
        tb = (tuned or tune or {}).get("tblock", 2)
        w16 = (tuned or tune or {}).get("tb16", 0)
        tile = "64 x 64" if (tuned or tune or {}).get("tb_narrow", 0) else "128 x 32"
        kern = (wl["kernel"] if steps_per_launch < 1.5 else
                "heat_tb2_kernel (radius 2, two time steps per launch, 64 x 64-cell tiles)" if wl["D"] == 2 else
                "heat2_kernel (two time steps per launch)" if tb == 2 and not w16 else
                f"heat_tb_kernel<{tb}> ({tb} time steps per launch, {tile}-cell tiles)")
        roof = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": profiled_traffic(args.workload, tb),
                "peak_source": peak_src, "kernel": kern,
                "algorithmic_bytes_per_launch": int(algo), "time_steps_per_launch": steps_per_launch,
                "avg_launch_ms": round(per_launch_ms, 4)}
    elif wl["model"] == 2:
        algo = wl["bytes_per_cell"] * cells * n
        achieved = algo / (ms / 1000.0) / 1e9
        roof = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": profiled_traffic(args.workload),
                "peak_source": peak_src, "kernel": wl["kernel"],
                "note": "whole-step average incl. halo exchanges; the 33.5 MB working set is L2-resident"}
    else:
        algo = wl["bytes_per_cell"] * cells * n
        achieved = algo / (ms / 1000.0) / 1e9
        kern = "eqwp_stag_fused" if tune.get("eqwp_fused") and wl["model"] == 4 else wl["kernel"]
        roof = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": profiled_traffic(args.workload),
                "peak_source": peak_src, "kernel": kern,
                "note": "whole-step average (stages and halo exchanges) over the algorithmic bytes "
                        "of one step"}

    # ---- parity of the timed schedule against the oracle (after timing)
    parity = parity_sample(d, wl, host) if rank == 0 else None

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        v, kind, cores, sample = cpu_sample(wl, budget_s=10.0)
        cpu = {"value": round(v, 4), "unit": "GLUPS", "cores": cores, "kind": kind, "sample": sample}

    line = None
    if rank == 0:
        line = {"metric": "GLUPS", "value": round(value, 3), "unit": "GLUPS", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "u8" if wl["model"] == 2 else "f32",
                "data": "synthetic (seeded U[0,1) / Bernoulli(0.3) / layered model)",
                "config": {**config_of(args, wl), **({"autotuned": tuned} if tuned else {})},
                "e2e": ({"value": round(e2e_val, 3), "unit": "GLUPS", "h2d_bytes_per_step": h2d,
                         "d2h_bytes_per_step": d2h} if e2e_val is not None else None),
                "gpu_launches": int(launches),
                "roofline": roof, "cpu_baseline": cpu, "clocks": clk, "parity": parity}
    d.close()
    return line


def profiled_traffic(workload, tblock=None):
    """DRAM bytes per launch of the dominant kernel from an ncu capture
    (profiles/traffic.json), keyed by workload and, for the heat sweeps that
    take several steps per launch, by "<workload>@tb<T>"."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(p):
        try:
            t = json.load(open(p))
            if tblock is not None and f"{workload}@tb{tblock}" in t:
                return t[f"{workload}@tb{tblock}"]
            return t.get(workload) if tblock in (None, 2) else None
        except Exception:
            return None
    return None


def run_workload(args, name):
    wl = WORKLOADS[name]
    a = argparse.Namespace(**{**vars(args), "workload": name})
    if wl["model"] == 5:
        return run_batch(a, wl)
    if wl["model"] == 6:
        return run_adjoint(a, wl)
    if wl["model"] == 7:
        return run_eqwp_batch(a, wl)
    return run_ours(a, wl)


# the BASELINE configurations other than the headline, carried under
# "secondary" by the default one-GPU run so that one invocation measures them
# all on the same box: each with its own value, roofline fraction, clocks and
# parity figure
SECONDARY = ("heat_128", "gol_256", "eqwp_stag", "heat4_512", "batch64", "eqwp_batch16", "adjoint256")


def compact(line):
    if line is None:
        return None
    roof = line.get("roofline") or {}
    cfg = line.get("config") or {}
    keep = ("autotuned", "batched_over_sequential", "sequential_plain_glups", "gradient_over_forward",
            "forward_ms", "gradient_ms", "time_steps_per_step", "env", "blocks", "R", "D", "l2")
    return {"value": line["value"], "unit": line["unit"], "ms_per_step": line["ms_per_step"],
            "steps": line["steps"], "warmup": line["warmup"],
            "e2e": (line.get("e2e") or {}).get("value"), "gpu_launches": line.get("gpu_launches"),
            "roofline_frac": roof.get("frac"), "roofline_kernel": roof.get("kernel"),
            "roofline_achieved_gbs": roof.get("achieved"), "clocks": line.get("clocks"),
            "parity": line.get("parity"), "config": {k: cfg[k] for k in keep if k in cfg}}


def main():
    args = parse()
    wl = WORKLOADS[args.workload]
    if args.impl == "reference":
        run_reference(args, wl)
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    line = run_workload(args, args.workload)
    if line is not None and world == 1 and args.secondary and args.workload == "heat1_512" and not args.tune:
        sec = {}
        short = argparse.Namespace(**{**vars(args), "steps": min(args.steps, 3), "warmup": 3,
                                      "no_cpu_baseline": True})
        for name in SECONDARY:
            try:
                sec[name] = compact(run_workload(short, name))
            except Exception as e:      # a secondary never takes the headline down
                sec[name] = {"error": str(e)[:300]}
        line["secondary"] = sec
    if line is not None:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        if dist.is_initialized():
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
