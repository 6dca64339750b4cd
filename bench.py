"""Benchmark: batched mixed-precision SBE + PSTD wire-steps/s on GB300.

Workload (default, "multiwire"): 32 identical GaAs-like quantum wires spaced
100 nm apart along a 1-D PSTD grid of Nx = 16384 cells of 10 nm (background
epsr = 12.9, absorbing layers of 128 cells), Nk = 512 k points per wire
(|k| <= 3e9 1/m, Nr = 1026), T = 300 K, Coulomb Hartree-Fock + screening +
LO-phonon relaxation + diagonal and off-diagonal dephasing.  The field is a
Gaussian pulse E0 = 5e7 V/m, tau = 50 fs, hbar w0 = Eg + 20 meV, launched by a
current sheet 2.5 um left of the array and already in flight at step 0 (its peak
at the array centre).  One step = one coupled step: field sampled onto every
wire, H update, RK4 step of every wire (dt = 0.05 fs: 4 RHS evaluations,
relaxation, charge normalisation, sources), sources deposited on the grid,
polarisation current, E update, longitudinal Ex.

value     : wire-steps/s of the mixed path (tcgen05 FP16 hi/lo x3, FP32 accumulate,
            FP64 state) through CoupledLine.step with device-resident state.
e2e       : the same call with the grid field (Ex, Ey, Ez) copied in from pinned
            host memory and the grid sources (Px, Py, Pz, Rho) read back every step.
fp64_gpu  : the plain FP64 GPU path on the same state (the metric's denominator).
roofline  : commutator GEMM launches (the dominant kernel), CUDA events around
            each launch inside the timed region.
cpu_baseline : the NumPy FP64 restatement (oracle) of one wire-step of the same
            workload on the host cores.

--impl reference prints the reference arm: the CPU implementation of the path
(the oracle restatement; the reference's own Numba path is not installable
here), one wire-step of the same workload per step.
"""

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

HBAR = 1.0545718176461565e-34
E0C = 1.602176634e-19
ME0 = 9.1093837139e-31
C0 = 299792458.0

WORKLOADS = {
    "multiwire": dict(nw=32, nk=512, kmax=3e9, temp=300.0, E0=5e7, tau=50e-15, det=20e-3,
                      dt=0.05e-15, spacing=100e-9, nx=16384, dx=10e-9, n_abc=128,
                      abc=0.05, x_src=-2.5e-6),
    # the same wires, fewer of them: the case the kernel-level profiles are taken on
    "profile": dict(nw=8, nk=512, kmax=3e9, temp=300.0, E0=5e7, tau=50e-15, det=20e-3,
                    dt=0.05e-15, spacing=100e-9, nx=16384, dx=10e-9, n_abc=128,
                    abc=0.05, x_src=-2.5e-6),
    # 16 wires: state matrices larger than L2 (201 MB in FP64), a few GB on the device
    "profile16": dict(nw=16, nk=512, kmax=3e9, temp=300.0, E0=5e7, tau=50e-15, det=20e-3,
                      dt=0.05e-15, spacing=100e-9, nx=16384, dx=10e-9, n_abc=128,
                      abc=0.05, x_src=-2.5e-6),
}

# Uneven sweep of independent wires in a local field: 512 wires drawn with
# numpy default_rng(3): Nk from {64, 96, 128, 192, 256, 384, 512} with weights
# proportional to 1/Nk, E0 log-uniform in [1e5, 1e8] V/m, detuning hbar w0 - Eg
# uniform in [-30, 100] meV, tau uniform in [30, 300] fs, T uniform in [10, 300] K;
# RK4 dt = 0.1 fs; each wire's pulse peaks at t = 2 tau from t = 0.
SWEEP = dict(nw=512, nks=(64, 96, 128, 192, 256, 384, 512), kmax=3e9, dt=0.1e-15, seed=3)

# Wires along z on a 3-D grid: 256 x 128 x 128 cells of 20 nm, 64 wires of Nk = 1024
# at (x, y) drawn with numpy default_rng(4) in the central 60 % of the x-y
# cross-section, a Gaussian beam (waist 1 um, polarised along y) E0 = 2e7 V/m, tau =
# 80 fs, hbar w0 = Eg + 30 meV launched along x by a current sheet next to the left
# absorbing layer and already in flight at step 0 (its peak at x = 0), RK4 and field
# step dt = 0.02 fs, T = 77 K.
GRID3 = dict(n=(256, 128, 128), d=20e-9, n_abc=(16, 8, 8), abc=0.05, nw=64, nk=1024, kmax=3e9,
             E0=2e7, tau=80e-15, det=30e-3, dt=0.02e-15, waist=1e-6, temp=77.0, seed=4,
             src_cell=24)

MAT = dict(me=0.067 * ME0, mh=0.45 * ME0, gap=1.52 * E0C, HO=100e-3 * E0C, Delta0=6e-9,
           gam_e=1e12, gam_h=1e12, gam_eh=1e12, epsr=12.9, Oph=36e-3 * E0C / HBAR,
           Gph=3e-3 * E0C / HBAR)
FLAGS = dict(Optics=True, Excitons=True, EHs=False, Screened=True, Phonon=True, DCTrans=False,
             LF=True, FreePot=False, DiagDph=True, OffDiagDph=True, Recomb=False)
METRIC = "SBE wire-steps/s: batched mixed-prec vs plain FP64 GPU at ≤1e-6 rel err"
# dram__bytes_read.sum + dram__bytes_write.sum of the commutator launches of one RHS
# evaluation (dP with the hi*lo + lo*hi products of W and V: 1070.4 + 171.8 MB; the
# hi*hi products of W and V in four K parts added to those: 404.6 + 100.0 MB),
# 32 wires x Nk = 512 (ncu, one timed coupled step), per wire
TRAFFIC_PER_EVAL_WIRE = (1070.4e6 + 171.8e6 + 404.6e6 + 100.0e6) / 32


def wire_L(nk, kmax):
    return np.pi / (kmax / (nk / 2 - 0.5))


def pulse(t, wl):
    w0 = (MAT["gap"] + wl["det"] * E0C) / HBAR
    return wl["E0"] * np.exp(-t * t / wl["tau"] ** 2) * np.cos(w0 * t)


def wire_positions(wl):
    return (np.arange(wl["nw"]) - (wl["nw"] - 1) / 2.0) * wl["spacing"]


def w0_of(wl):
    return (MAT["gap"] + wl["det"] * E0C) / HBAR


def incident_state(wl, x, x_src, t, dt):
    """Grid fields of the pulse a current sheet at x_src has emitted since t = -inf:
    Ey(x, t) = E_inc(t - |x - x_src| / v), Hz(x, t - dt/2) = sign(x - x_src) Ey / eta."""
    v = C0 / np.sqrt(MAT["epsr"])
    eta = np.sqrt(1.25663706127e-06 / (8.8541878188e-12 * MAT["epsr"]))
    d = np.abs(x - x_src)
    E = np.zeros((2, len(x)), complex)
    H = np.zeros((2, len(x)), complex)
    E[0] = pulse(t - d / v, wl)
    H[0] = np.sign(x - x_src) * pulse(t - dt / 2 - d / v, wl) / eta
    return E, H


def env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def dist_init(world, backend=None):
    """Process group of a torchrun launch (one rank per GPU, each stepping its own
    replica of the wire batch): NCCL where the ranks have GPUs, gloo where they have
    none or where backend says so (the CPU test of this logic).  None for a single
    process."""
    if world <= 1:
        return None
    import torch
    import torch.distributed as dist
    if not dist.is_initialized():
        dist.init_process_group(backend or ("nccl" if torch.cuda.is_available() else "gloo"))
    return dist


def max_over_ranks(dist, ms):
    """The job's time: the largest of the ranks' times, returned on every rank."""
    if dist is None:
        return ms
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(ms)], device=dev, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(world, nw, steps, ms):
    """Whole-job wire-steps/s: each of the world ranks steps nw wires (weak scaling)
    steps times in ms milliseconds (the slowest rank's time)."""
    return world * nw * steps / (ms / 1e3)


# ---------------------------------------------------------------------------
# CPU arm (the oracle restatement) -------------------------------------------


def cpu_wire_steps(wl, nsteps, warm):
    """Time nsteps RK4 wire-steps of one wire of the workload with the oracle."""
    from oracle import sbe_oracle as O
    nk = wl["nk"]
    L = wire_L(nk, wl["kmax"])
    w = O.Wire(nk, L, MAT, FLAGS, wl["temp"])
    fe = O.fermi(w.c["Ee"] + MAT["gap"] / 2.0, wl["temp"])
    P = np.zeros((nk, nk), complex)
    C = np.diag(fe).astype(complex)
    D = C.copy()
    wk = O.fftg(w.window)
    z = np.zeros_like(wk)
    t = -2 * wl["tau"]
    dt = wl["dt"]
    times = []
    for i in range(warm + nsteps):
        e0 = pulse(t, wl)
        e1 = pulse(t + dt, wl)
        t0 = time.perf_counter()
        P, C, D = w.rk4_step(P, C, D, [z, e0 * wk, z], [z, (e1 - e0) * wk, z], dt, 1)[:3]
        times.append(time.perf_counter() - t0)
        t += dt
    return times[warm:]


def sweep_wires():
    """Per-wire Nk, E0 (V/m), detuning (J), tau (s) and T (K) of the sweep workload."""
    rng = np.random.default_rng(SWEEP["seed"])
    nks = np.array(SWEEP["nks"])
    p = (1.0 / nks) / np.sum(1.0 / nks)
    n = SWEEP["nw"]
    nk = rng.choice(nks, size=n, p=p)
    E0 = 10.0 ** rng.uniform(5.0, 8.0, n)
    det = rng.uniform(-30e-3, 100e-3, n) * E0C
    tau = rng.uniform(30e-15, 300e-15, n)
    temp = rng.uniform(10.0, 300.0, n)
    return nk, E0, det, tau, temp


def sweep_fields(t, E0, det, tau):
    """Local field of every wire at time t: E0 exp(-((t - 2 tau)/tau)^2) cos(w0 (t - 2 tau))."""
    w0 = (MAT["gap"] + det) / HBAR
    x = t - 2.0 * tau
    return E0 * np.exp(-(x / tau) ** 2) * np.cos(w0 * x)


def sweep_config():
    nk, _, _, _, _ = sweep_wires()
    counts = {int(k): int(np.sum(nk == k)) for k in SWEEP["nks"]}
    return {"workload": f"{SWEEP['nw']} independent GaAs-like wires in a local field, Nk drawn "
                        "from {64,96,128,192,256,384,512} with weights 1/Nk (default_rng(3)), "
                        "E0 log-uniform 1e5-1e8 V/m, detuning U[-30,100] meV, tau U[30,300] fs, "
                        "T U[10,300] K, RK4 dt=0.10 fs",
            "wires": SWEEP["nw"], "nk_counts": counts,
            "flags": " ".join(k for k, v in FLAGS.items() if v),
            "integrator": "RK4 (coefficients frozen per step) + reference relaxation/normalisation",
            "l2": "inputs larger than L2 (FP64 state %.0f MB)" %
                  (3 * 16 * float(np.sum(nk.astype(float) ** 2)) / 1e6)}


def cpu_sweep_rate():
    """CPU wire-steps/s of the sweep from one timed oracle RK4 step of one wire of each Nk
    (the wire-step time of the workload = sum over its wires of the time of their Nk)."""
    from oracle import sbe_oracle as O
    nk_all, E0, det, tau, temp = sweep_wires()
    per_nk = {}
    for nk in SWEEP["nks"]:
        w = int(np.nonzero(nk_all == nk)[0][0])
        L = wire_L(nk, SWEEP["kmax"])
        wire = O.Wire(int(nk), L, MAT, FLAGS, float(temp[w]))
        fe = O.fermi(wire.c["Ee"] + MAT["gap"] / 2.0, float(temp[w]))
        P = np.zeros((nk, nk), complex)
        C = np.diag(fe).astype(complex)
        wk = O.fftg(wire.window)
        z = np.zeros_like(wk)
        e0 = sweep_fields(0.0, E0[w], det[w], tau[w])
        t0 = time.perf_counter()
        wire.rk4_step(P, C, C.copy(), [z, e0 * wk, z], [z, 0 * wk, z], SWEEP["dt"], 1)
        per_nk[int(nk)] = time.perf_counter() - t0
    total = float(sum(per_nk[int(k)] for k in nk_all))
    return SWEEP["nw"] / total, per_nk


def reference_timing():
    """The reference's own pure-Python step (SBESolver + QWCalculator, Nk = 64 local
    field) as timed by oracle/time_reference.py where the reference source is available
    (it is not on the GPU host): the recorded figures with the host they come from."""
    p = os.path.join(ROOT, "oracle", "reference_timing.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        d = json.load(f)
    d["note"] = "measured by oracle/time_reference.py on the host named here, not in this run"
    return d


def reference_arm(args, wl):
    rank, world, local = env()
    if rank != 0:
        return
    if wl is None:
        v, per_nk = cpu_sweep_rate()
        line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "wire-steps/s",
                "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": 1e3 * SWEEP["nw"] / v, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": sweep_config(),
                "cpu_baseline": {"value": v, "unit": "wire-steps/s", "cores": os.cpu_count(),
                                 "kind": "port",
                                 "sample": "one RK4 step of one wire of each Nk (NumPy FP64 "
                                           "restatement), summed over the workload's wires: "
                                           + ", ".join(f"Nk={k}: {t:.3f} s"
                                                       for k, t in per_nk.items())},
                "e2e": {"value": v, "unit": "wire-steps/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return
    times = cpu_wire_steps(wl, args.steps, args.warmup)
    tot = sum(times)
    v = len(times) / tot
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "wire-steps/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * tot / len(times), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config_of(wl),
            "cpu_baseline": {"value": v, "unit": "wire-steps/s", "cores": os.cpu_count(),
                             "kind": "port",
                             "sample": f"one wire of the {wl['nw']}-wire batch, Nk={wl['nk']}, "
                                       f"{len(times)} RK4 steps (NumPy FP64 restatement; BLAS "
                                       "matmuls multi-threaded, O(Nk^3) sums single-threaded)"},
            "e2e": {"value": v, "unit": "wire-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def config_of(wl):
    return {"workload": f"{wl['nw']} wires x Nk={wl['nk']} GaAs-like quantum wires every "
                        f"{wl['spacing']*1e9:.0f} nm on a 1-D PSTD grid Nx={wl['nx']} "
                        f"dx={wl['dx']*1e9:.0f} nm, pulse E0={wl['E0']:.0e} V/m "
                        f"tau={wl['tau']*1e15:.0f} fs, T={wl['temp']:.0f} K, "
                        f"RK4 dt={wl['dt']*1e15:.2f} fs",
            "wires": wl["nw"], "nk": wl["nk"], "nr": 2 * wl["nk"] + 2, "nx": wl["nx"],
            "flags": " ".join(k for k, v in FLAGS.items() if v),
            "integrator": "RK4 (coefficients frozen per step) + reference relaxation/normalisation",
            "l2": "inputs larger than L2 (FP64 state 403 MB, FP16 operand planes 1.9 GB per stage)"}


# ---------------------------------------------------------------------------
# GPU arm ----------------------------------------------------------------------


class ClockSampler:
    def __init__(self, idx, path):
        self.p = None
        self.path = path
        try:
            self.f = open(path, "w")
            self.p = subprocess.Popen(
                ["nvidia-smi", f"--id={idx}",
                 "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,"
                 "clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "50"], stdout=self.f,
                stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None
        # nvidia-smi takes a while to start: wait (up to 5 s) for its first sample so
        # that the samples cover the timed region that follows
        t0 = time.time()
        while self.p is not None and time.time() - t0 < 5.0:
            try:
                if os.path.getsize(path) > 0:
                    break
            except OSError:
                pass
            time.sleep(0.02)

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.close()
        with open(self.path) as f:
            return clock_summary(f)


def clock_summary(lines):
    """Median SM clock, maximum clock and the throttle reasons seen in nvidia-smi samples
    (csv, noheader, nounits: index, clocks.sm, clocks.max.sm, power.draw, active mask,
    then hw_slowdown, hw_thermal_slowdown, sw_thermal_slowdown, sw_power_cap as
    "Active" / "Not Active"); lines that are not samples are skipped."""
    sm, smax, reasons = [], None, set()
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    for ln in lines:
        parts = [x.strip() for x in ln.split(",")]
        if len(parts) < 9:
            continue
        try:
            sm.append(float(parts[1]))
            smax = float(parts[2])
        except ValueError:
            continue
        for nm, v in zip(names, parts[5:9]):
            if v.lower().startswith("active"):
                reasons.add(nm)
    return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax,
            "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d, "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def gpu_arm(args, wl):
    import torch
    import __graft_entry__ as ge
    rank, world, local = env()
    dist = dist_init(world)
    torch.cuda.set_device(local)
    ge.build()
    from pulsesuite_gb300 import _lib
    from pulsesuite_gb300.pstd import CoupledLine, Pstd1D, SheetSource
    from pulsesuite_gb300.wires import WireContext, WireSpec

    nw, nk = wl["nw"], wl["nk"]
    L = wire_L(nk, wl["kmax"])
    specs = [WireSpec(nk=nk, L=L, temp=wl["temp"], wire_index=w + 1, flags=dict(FLAGS), **MAT)
             for w in range(nw)]
    ctx = WireContext(specs)
    prec = _lib.PREC_MIXED if args.precision == "mixed" else _lib.PREC_FP64
    nx, dx, dt = wl["nx"], wl["dx"], wl["dt"]
    grid = Pstd1D(nx, dx, MAT["epsr"], n_abc=wl["n_abc"], abc_strength=wl["abc"])
    x = grid.x.cpu().numpy()
    i_src = int(np.argmin(np.abs(x - wl["x_src"])))
    x_src = float(x[i_src])
    v = C0 / np.sqrt(MAT["epsr"])
    t_start = (0.0 - x_src) / v                 # pulse peak at the array centre at step 0
    line = CoupledLine(ctx, grid, wire_positions(wl),
                       source=SheetSource(index=i_src, E0=wl["E0"], tau=wl["tau"],
                                          w0=w0_of(wl), tpeak=0.0),
                       t0=t_start, longitudinal=True)
    E0h, H0h = incident_state(wl, x, x_src, t_start, dt)
    # GEMM tiles of the mixed path from the autotuner (cached per device and shape)
    cache = args.tile_cache or os.path.join(tempfile.gettempdir(), "sbe_tiles.json")
    tiles = ctx.autotune(cache) if prec == _lib.PREC_MIXED else []

    fe = 1.0 / (np.exp((ctx.table(0, "Ee").cpu().numpy() + MAT["gap"] / 2.0) / 1.380649e-23
                       / wl["temp"]) + 1.0)

    def fresh():
        d = np.diag(fe).astype(complex)
        P = ctx.zeros_state()
        C = ctx.pack([d] * nw)
        D = ctx.pack([d] * nw)
        E = torch.as_tensor(E0h).cuda().contiguous()
        H = torch.as_tensor(H0h).cuda().contiguous()
        Ex = torch.zeros(nx, dtype=torch.complex128, device="cuda")
        return P, C, D, E, H, Ex

    st = fresh()
    line.reset()
    for _ in range(args.warmup):
        line.step(*st, dt, prec)
    torch.cuda.synchronize()

    # timed region: device-resident state, engine launches timed with events
    ctx.profile(True)
    for cat in range(4):
        ctx.profile_read(cat)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    # the raw nvidia-smi samples go to SBE_CLOCKS_DIR (default: the temp dir); the
    # JSON line carries their summary
    clk_dir = os.environ.get("SBE_CLOCKS_DIR", tempfile.gettempdir())
    clocks = ClockSampler(local, os.path.join(clk_dir, f"clocks_{rank}.csv"))
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record()
    torch.cuda.nvtx.range_push("timed_steps")   # ncu --nvtx-include timed_steps/
    for _ in range(args.steps):
        line.step(*st, dt, prec)
    torch.cuda.nvtx.range_pop()
    ev1.record()
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    clk = clocks.stop()
    if dist:
        ms = max_over_ranks(dist, ms)
        dist.barrier()
    prof = {cat: ctx.profile_read(cat) for cat in range(4)}
    ctx.profile(False)
    ctx.check()
    # the FP64 conservation check of the last timed step (read after the timed region)
    charge_imb = ctx.charge_imbalance()
    value = job_rate(world, nw, args.steps, ms)

    # CUDA graph of the same coupled step (launch count, replay time)
    graph = line.graph(*st, dt, prec)
    n_kernels = graph.kernels
    graph.launch()
    torch.cuda.synchronize()
    g0 = torch.cuda.Event(enable_timing=True)
    g1 = torch.cuda.Event(enable_timing=True)
    g0.record()
    for _ in range(args.steps):
        graph.launch()
    g1.record()
    torch.cuda.synchronize()
    graph_ms = g0.elapsed_time(g1) / args.steps
    graph.close()

    # PSTD field step alone (H and E updates of the 16384-cell grid)
    Et, Ht = st[3].clone(), st[4].clone()
    Jt = torch.zeros_like(Et)
    for _ in range(3):
        grid.step(Et, Ht, Jt, dt)
    p0 = torch.cuda.Event(enable_timing=True)
    p1 = torch.cuda.Event(enable_timing=True)
    p0.record()
    for _ in range(100):
        grid.step(Et, Ht, Jt, dt)
    p1.record()
    torch.cuda.synchronize()
    pstd_ms = p0.elapsed_time(p1) / 100

    # end to end: grid field (Ex, Ey, Ez) in from pinned host memory, grid sources
    # (Px, Py, Pz, Rho) back to pinned host memory, every step
    h_in = [torch.cat([st[5][None], st[3]]).cpu().pin_memory() for _ in range(args.steps)]
    h_out = torch.empty((4, nx), dtype=torch.complex128).pin_memory()
    Pg, rho = line.view("Pg"), line.view("rho")
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for i in range(args.steps):
        st[5].copy_(h_in[i][0], non_blocking=True)
        st[3].copy_(h_in[i][1:], non_blocking=True)
        line.step(*st, dt, prec)
        h_out[:3].copy_(Pg, non_blocking=True)
        h_out[3].copy_(rho, non_blocking=True)
    e1.record()
    torch.cuda.synchronize()
    e2e_ms = max_over_ranks(dist, e0.elapsed_time(e1))
    e2e_val = job_rate(world, nw, args.steps, e2e_ms)

    # RHS error of the mixed path against the FP64 path at the current state
    P, C, D = st[0], st[1], st[2]
    Ek_now = line.view("Ek").clone()
    r64 = ctx.rhs(P, C, D, Ek_now, _lib.PREC_FP64)
    rmx = ctx.rhs(P, C, D, Ek_now, _lib.PREC_MIXED)
    rhs_err = max(float(torch.linalg.norm(a - b) / torch.linalg.norm(b)) for a, b in zip(rmx, r64))
    field_peak = float(Ek_now.abs().max())

    # plain FP64 GPU path on the same state (a few steps: it is slow by design)
    fp64_ms = fp64_val = None
    n64 = max(1, args.fp64_steps)
    if not args.no_fp64:
        st64 = tuple(t.clone() for t in st)
        line.step(*st64, dt, _lib.PREC_FP64)
        torch.cuda.synchronize()
        f0e = torch.cuda.Event(enable_timing=True)
        f1e = torch.cuda.Event(enable_timing=True)
        f0e.record()
        for _ in range(n64):
            line.step(*st64, dt, _lib.PREC_FP64)
        f1e.record()
        torch.cuda.synchronize()
        fp64_ms = max_over_ranks(dist, f0e.elapsed_time(f1e) / n64)
        fp64_val = job_rate(world, nw, 1, fp64_ms)

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return

    peaks, pk_kind = measured_peaks()
    comm_ms, comm_n = prof[0]
    evals = 4 * args.steps                  # RHS evaluations in the timed region
    per_eval_s = comm_ms / evals / 1e3      # commutator GEMM time of one evaluation
    # algorithmic work of a1-a3 per RHS evaluation: dP, dC, dD as 12 complex Nk^3
    # products = 96 Nk^3 flop per wire
    useful = 96.0 * nk ** 3 * nw
    # executed per wire, in 2 Nk^3 real-product MMA chains: dP 4 complex terms x 4 real
    # products x 3 hi/lo terms = 48; W, V 2 complex terms each x 4 x (hi*lo, lo*hi) =
    # 32; their hi*hi products 16: 96 x 2 Nk^3 = 192 Nk^3
    executed = 192.0 * nk ** 3 * nw
    achieved = useful / per_eval_s / 1e12
    peak = peaks.get("bf16_tflops_sustained", 1700.0)
    roof = {"bound": "tensor", "kernel": "k_tc_gemm (commutator dP/dC/dD)", "achieved": achieved,
            "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
            "peak_kind": f"{pk_kind} bf16 dense sustained (fp16 dense has the same rate)",
            "executed_tflops": executed / per_eval_s / 1e12,
            "executed_frac": executed / per_eval_s / 1e12 / peak,
            "ms_per_rhs_eval": per_eval_s * 1e3, "launches": comm_n,
            "avg_launch_ms": comm_ms / max(comm_n, 1),
            "traffic": TRAFFIC_PER_EVAL_WIRE * nw,
            "traffic_note": "DRAM read+write bytes of the commutator launches of one RHS "
                            "evaluation: dram__bytes_read.sum + dram__bytes_write.sum of an ncu "
                            "capture of one timed step of the 32-wire case "
                            "(profiles/coupled_step_dram_multiwire_nk512.md), scaled by wires; "
                            "a constant of this file, refreshed with the profile",
            "flops_model": "algorithmic 96*Nk^3 per wire per RHS evaluation (dpdt/dCdt/dDdt as "
                           "12 complex Nk^3 products) over the summed CUDA-event time of the "
                           "evaluation's two commutator launches (dP with the hi*lo + lo*hi "
                           "products of W and V; the hi*hi products of W and V in K parts with "
                           "one accumulator per real product, added to them in order); executed "
                           "192*Nk^3 (dP 96, W and V cross terms 64, their hi*hi products 32); "
                           "step: 496*Nk^3 "
                           "algorithmic flop per wire-step (4 evaluations of a1-a3 and the "
                           "exchange and source products) over the step time",
            "step_tflops": 496.0 * nk ** 3 * value / 1e12,
            "step_frac": 496.0 * nk ** 3 * value / 1e12 / peak}
    other = {name: {"ms_per_step": prof[c][0] / args.steps, "launches": prof[c][1]}
             for c, name in ((1, "exchange_gemm"), (2, "source_gemm"), (3, "dephasing_fp32"))}
    other["pstd_field_step"] = {"ms_per_step": pstd_ms, "launches": 6}

    cpu = None
    if not args.no_cpu:
        ct = cpu_wire_steps(wl, 1, 0)
        cpu = {"value": 1.0 / ct[0], "unit": "wire-steps/s", "cores": os.cpu_count(),
               "kind": "port",
               "sample": f"one RK4 wire-step of one wire (Nk={nk}) of this workload, NumPy FP64 "
                         "restatement (BLAS matmuls multi-threaded, O(Nk^3) sums single-threaded)",
               "reference_python": reference_timing()}

    line_out = {"metric": METRIC, "value": value, "unit": "wire-steps/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "fp16x3-f32acc/f64" if prec == _lib.PREC_MIXED else "f64",
                "data": "synthetic", "config": config_of(wl), "precision": args.precision,
                "clocks": clk,
                "e2e": {"value": e2e_val, "unit": "wire-steps/s",
                        "h2d_bytes_per_step": int(3 * nx * 16),
                        "d2h_bytes_per_step": int(4 * nx * 16)},
                "gpu_launches": int(n_kernels * args.steps),
                "gpu_launches_per_step": int(n_kernels),
                "graph_replay_ms_per_step": graph_ms,
                "roofline": roof, "other_kernels": other, "tiles": tiles,
                "fp64_gpu": {"value": fp64_val, "unit": "wire-steps/s", "ms_per_step": fp64_ms,
                             "steps": n64},
                "speedup_vs_fp64_gpu": (value / fp64_val) if fp64_val else None,
                "rhs_rel_err_vs_fp64": rhs_err,
                "charge_imbalance": {"value": charge_imb,
                                     "what": "max over wires of |N_e - N_h| / mean found by the "
                                             "FP64 charge normalisation of the last timed step"},
                "wire_field_peak_k": field_peak,
                "cpu_baseline": cpu}
    print(json.dumps(line_out), flush=True)
    if dist:
        dist.destroy_process_group()


def sweep_arm(args):
    """The uneven sweep on the mixed path: one RK4 step of all 512 wires per step, the
    GEMMs of all Nk buckets in one persistent launch per kind, tiles from the
    autotuner."""
    import torch
    import __graft_entry__ as ge
    rank, world, local = env()
    dist = dist_init(world)
    torch.cuda.set_device(local)
    ge.build()
    from pulsesuite_gb300 import _lib
    from pulsesuite_gb300.wires import WireContext, WireSpec
    nk, E0, det, tau, temp = sweep_wires()
    nw, dt = SWEEP["nw"], SWEEP["dt"]
    specs = [WireSpec(nk=int(nk[w]), L=wire_L(int(nk[w]), SWEEP["kmax"]), temp=float(temp[w]),
                      wire_index=w + 1, flags=dict(FLAGS), **MAT) for w in range(nw)]
    t_ctx = time.perf_counter()
    ctx = WireContext(specs)
    t_ctx = time.perf_counter() - t_ctx
    prec = _lib.PREC_MIXED if args.precision == "mixed" else _lib.PREC_FP64
    cache = args.tile_cache or os.path.join(tempfile.gettempdir(), "sbe_tiles.json")
    t_tune = time.perf_counter()
    tiles = ctx.autotune(cache) if prec == _lib.PREC_MIXED else []
    t_tune = time.perf_counter() - t_tune

    def fresh():
        P = ctx.zeros_state()
        ds = []
        for w in range(nw):
            Ee = ctx.table(w, "Ee").cpu().numpy()
            x = np.minimum((Ee + MAT["gap"] / 2.0) / (1.380649e-23 * temp[w]), 700.0)
            ds.append(np.diag(1.0 / (np.exp(x) + 1.0)).astype(complex))
        return P, ctx.pack(ds), ctx.pack(ds)

    nsteps = args.warmup + args.steps
    # per-step field amplitudes of every wire (host), resident on the device for `value`
    amps = np.stack([sweep_fields(n * dt, E0, det, tau) for n in range(nsteps + 1)])
    e0_dev = torch.as_tensor(amps[:-1]).cuda()
    de_dev = torch.as_tensor(amps[1:] - amps[:-1]).cuda()
    P, C, D = fresh()
    Ek0, dEk = ctx.zeros_r(3), ctx.zeros_r(3)
    src = ctx.zeros_r(5)
    for n in range(args.warmup):
        ctx.local_field(e0_dev[n], de_dev[n], 1, Ek0, dEk)
        ctx.rk4_step(P, C, D, Ek0, dEk, dt, src, prec)
    torch.cuda.synchronize()
    # timed region: one step of all wires per step (direct calls, engine launches timed
    # with events); the same step as a CUDA graph is timed after it
    ctx.profile(True)
    for cat in range(4):
        ctx.profile_read(cat)
    clk_dir = os.environ.get("SBE_CLOCKS_DIR", tempfile.gettempdir())
    clocks = ClockSampler(local, os.path.join(clk_dir, f"clocks_sweep_{rank}.csv"))
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    ev0.record()
    torch.cuda.nvtx.range_push("timed_steps")   # ncu --nvtx-include timed_steps/
    for n in range(args.warmup, nsteps):
        ctx.local_field(e0_dev[n], de_dev[n], 1, Ek0, dEk)
        ctx.rk4_step(P, C, D, Ek0, dEk, dt, src, prec)
    torch.cuda.nvtx.range_pop()
    ev1.record()
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    clk = clocks.stop()
    prof = {cat: ctx.profile_read(cat) for cat in range(4)}
    ctx.profile(False)
    ctx.check()
    graph = ctx.rk4_graph(P, C, D, Ek0, dEk, dt, src, prec)
    n_kernels = graph.kernels
    g0 = torch.cuda.Event(enable_timing=True)
    g1 = torch.cuda.Event(enable_timing=True)
    g0.record()
    for n in range(args.warmup, nsteps):
        ctx.local_field(e0_dev[n], de_dev[n], 1, Ek0, dEk)
        graph.launch()
    g1.record()
    torch.cuda.synchronize()
    graph_ms = g0.elapsed_time(g1) / args.steps
    if dist:
        ms = max_over_ranks(dist, ms)
    value = job_rate(world, nw, args.steps, ms)

    # end to end: the step's field amplitudes from pinned host memory, the wires'
    # real-space sources (Px, Py, Pz, re, rh) back to pinned host memory every step
    h_e0 = torch.as_tensor(amps[:-1]).pin_memory()
    h_de = torch.as_tensor(amps[1:] - amps[:-1]).pin_memory()
    d_e0 = torch.empty(nw, dtype=torch.float64, device="cuda")
    d_de = torch.empty(nw, dtype=torch.float64, device="cuda")
    h_src = torch.empty(src.numel(), dtype=torch.complex128).pin_memory()
    torch.cuda.synchronize()
    e0e = torch.cuda.Event(enable_timing=True)
    e1e = torch.cuda.Event(enable_timing=True)
    e0e.record()
    for n in range(args.warmup, nsteps):
        d_e0.copy_(h_e0[n], non_blocking=True)
        d_de.copy_(h_de[n], non_blocking=True)
        ctx.local_field(d_e0, d_de, 1, Ek0, dEk)
        graph.launch()
        h_src.copy_(src, non_blocking=True)
    e1e.record()
    torch.cuda.synchronize()
    e2e_ms = max_over_ranks(dist, e0e.elapsed_time(e1e))
    graph.close()

    # RHS error against FP64 at the current state (every wire)
    ctx.local_field(e0_dev[nsteps - 1], None, 1, Ek0, None)
    r64 = ctx.rhs(P, C, D, Ek0, _lib.PREC_FP64)
    rmx = ctx.rhs(P, C, D, Ek0, _lib.PREC_MIXED)
    errs = []
    for a, b in zip(rmx, r64):
        for w in range(nw):
            bw = ctx.mat(b, w)
            nb = float(torch.linalg.norm(bw))
            if nb > 0:
                errs.append(float(torch.linalg.norm(ctx.mat(a, w) - bw)) / nb)
    rhs_err = max(errs)

    # the plain FP64 GPU path on the same wires and state
    fp64_ms = fp64_val = None
    if not args.no_fp64:
        st64 = (P.clone(), C.clone(), D.clone())
        s64 = ctx.zeros_r(5)
        ctx.rk4_step(*st64, Ek0, dEk, dt, s64, _lib.PREC_FP64)
        torch.cuda.synchronize()
        f0 = torch.cuda.Event(enable_timing=True)
        f1 = torch.cuda.Event(enable_timing=True)
        n64 = max(1, args.fp64_steps)
        f0.record()
        for _ in range(n64):
            ctx.rk4_step(*st64, Ek0, dEk, dt, s64, _lib.PREC_FP64)
        f1.record()
        torch.cuda.synchronize()
        fp64_ms = max_over_ranks(dist, f0.elapsed_time(f1) / n64)
        fp64_val = job_rate(world, nw, 1, fp64_ms)
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    peaks, pk_kind = measured_peaks()
    peak = peaks.get("bf16_tflops_sustained", 1700.0)
    sum_nk3 = float(np.sum(nk.astype(float) ** 3))
    comm_ms, comm_n = prof[0]
    per_eval_s = comm_ms / (4 * args.steps) / 1e3
    achieved = 96.0 * sum_nk3 / per_eval_s / 1e12
    step_tflops = 496.0 * sum_nk3 * (args.steps / (ms / 1e3)) / 1e12
    cpu = None
    if not args.no_cpu:
        v, per_nk = cpu_sweep_rate()
        cpu = {"value": v, "unit": "wire-steps/s", "cores": os.cpu_count(), "kind": "port",
               "sample": "one RK4 step of one wire of each Nk (NumPy FP64 restatement), summed "
                         "over the workload's wires"}
    line_out = {"metric": METRIC, "value": value, "unit": "wire-steps/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "fp16x3-f32acc/f64" if prec == _lib.PREC_MIXED else "f64",
                "data": "synthetic", "config": sweep_config(), "precision": args.precision,
                "clocks": clk,
                "e2e": {"value": job_rate(world, nw, args.steps, e2e_ms), "unit": "wire-steps/s",
                        "h2d_bytes_per_step": int(2 * 8 * nw),
                        "d2h_bytes_per_step": int(src.numel() * 16)},
                "gpu_launches": int((n_kernels + 1) * args.steps),
                "gpu_launches_per_step": int(n_kernels + 1),
                "graph_replay_ms_per_step": graph_ms,
                "roofline": {"bound": "tensor", "kernel": "k_tc_gemm (commutator dP/dC/dD)",
                             "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                             "frac": achieved / peak,
                             "peak_kind": f"{pk_kind} bf16 dense sustained",
                             "ms_per_rhs_eval": per_eval_s * 1e3, "launches": comm_n,
                             "traffic": None,
                             "step_tflops": step_tflops, "step_frac": step_tflops / peak,
                             "flops_model": "96*sum(Nk^3) per RHS evaluation over the commutator "
                                            "launches; step: 496*sum(Nk^3) per step"},
                "other_kernels": {name: {"ms_per_step": prof[c][0] / args.steps,
                                         "launches": prof[c][1]}
                                  for c, name in ((1, "exchange_gemm"), (2, "source_gemm"),
                                                  (3, "dephasing_fp32"))},
                "tiles": tiles, "autotune_s": t_tune, "ctx_create_s": t_ctx,
                "fp64_gpu": {"value": fp64_val, "unit": "wire-steps/s", "ms_per_step": fp64_ms},
                "speedup_vs_fp64_gpu": (value / fp64_val) if fp64_val else None,
                "rhs_rel_err_vs_fp64": rhs_err,
                "cpu_baseline": cpu}
    print(json.dumps(line_out), flush=True)
    if dist:
        dist.destroy_process_group()


def grid3_config():
    g = GRID3
    return {"workload": f"{g['nw']} GaAs-like wires of Nk={g['nk']} along z at seeded (x, y) in the "
                        f"central 60% of a {g['n'][0]}x{g['n'][1]}x{g['n'][2]} 3-D PSTD grid of "
                        f"{g['d']*1e9:.0f} nm, Gaussian beam E0={g['E0']:.0e} V/m "
                        f"tau={g['tau']*1e15:.0f} fs hbar w0=Eg+{g['det']*1e3:.0f} meV, "
                        f"T={g['temp']:.0f} K, RK4 dt={g['dt']*1e15:.2f} fs",
            "wires": g["nw"], "nk": g["nk"], "grid": list(g["n"]),
            "flags": " ".join(k for k, v in FLAGS.items() if v),
            "field": "3-D PSTD, six c128 components, FP32 transforms, FP64 fields",
            "l2": "inputs larger than L2 (FP64 wire state 3.2 GB, fields 403 MB)"}


def grid3_field_arm(args):
    """The 3-D field step alone on the 256 x 128 x 128 grid (FP32 transforms, a fixed
    current): steps/s and achieved HBM GB/s (the case the FFT-pass profiles use)."""
    import torch
    import __graft_entry__ as ge
    torch.cuda.set_device(env()[2])
    ge.build()
    from pulsesuite_gb300.pstd import Pstd3D
    g3 = GRID3
    n, d = g3["n"], g3["d"]
    grid = Pstd3D(n, (d, d, d), MAT["epsr"], n_abc=g3["n_abc"], abc_strength=g3["abc"],
                  fp32_work=args.precision == "mixed")
    gen = torch.Generator(device="cuda").manual_seed(0)
    E = torch.randn((3,) + n, dtype=torch.complex128, device="cuda", generator=gen) * 1e6
    H = torch.randn((3,) + n, dtype=torch.complex128, device="cuda", generator=gen) * 1e3
    J = torch.randn((3,) + n, dtype=torch.complex128, device="cuda", generator=gen) * 1e9
    dt = g3["dt"]
    for _ in range(args.warmup):
        grid.step(E, H, J, dt)
    torch.cuda.synchronize()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(args.steps):
        grid.step(E, H, J, dt)
    b.record()
    torch.cuda.synchronize()
    ms = a.elapsed_time(b) / args.steps
    peaks, pk_kind = measured_peaks()
    N = n[0] * n[1] * n[2]
    gbs = N * 240 / (ms / 1e3) / 1e9
    print(json.dumps({"workload": "3-D field step alone, 256x128x128 x 20 nm, six c128 components",
                      "precision": args.precision, "steps": args.steps, "ms_per_step": ms,
                      "achieved_gbs": gbs, "peak_gbs": peaks.get("hbm_gbs"), "peak_kind": pk_kind,
                      "frac": gbs / peaks.get("hbm_gbs", 6800.0),
                      "bytes_model": "E, H read and written, J read: 240 B per point"}), flush=True)


def grid3_arm(args):
    """Config 4: 64 wires of Nk = 1024 coupled to the 3-D grid; value = wire-steps/s of
    the coupled step (mixed path); the field step alone is timed for its HBM roofline."""
    import torch
    import __graft_entry__ as ge
    if args.field_only:
        grid3_field_arm(args)
        return
    rank, world, local = env()
    dist = dist_init(world)
    torch.cuda.set_device(local)
    ge.build()
    from pulsesuite_gb300 import _lib
    from pulsesuite_gb300.pstd import CoupledGrid3, Pstd3D, SheetSource
    from pulsesuite_gb300.wires import WireContext, WireSpec
    g3 = GRID3
    n, d, nw, nk, dt = g3["n"], g3["d"], g3["nw"], g3["nk"], g3["dt"]
    rng = np.random.default_rng(g3["seed"])
    Lx, Ly = (n[0] - 1) * d, (n[1] - 1) * d
    wxy = np.stack([rng.uniform(-0.3 * Lx, 0.3 * Lx, nw), rng.uniform(-0.3 * Ly, 0.3 * Ly, nw)], 1)
    L = wire_L(nk, g3["kmax"])
    specs = [WireSpec(nk=nk, L=L, temp=g3["temp"], wire_index=w + 1, flags=dict(FLAGS), **MAT)
             for w in range(nw)]
    t_ctx = time.perf_counter()
    ctx = WireContext(specs)
    t_ctx = time.perf_counter() - t_ctx
    prec = _lib.PREC_MIXED if args.precision == "mixed" else _lib.PREC_FP64
    grid = Pstd3D(n, (d, d, d), MAT["epsr"], n_abc=g3["n_abc"], abc_strength=g3["abc"],
                  fp32_work=prec == _lib.PREC_MIXED)
    x = grid.x[0].cpu().numpy()
    y = grid.x[1].cpu().numpy()
    z = grid.x[2].cpu().numpy()
    i_src = g3["n_abc"][0] + g3["src_cell"]
    x_src = float(x[i_src])
    v = C0 / np.sqrt(MAT["epsr"])
    w0 = (MAT["gap"] + g3["det"] * E0C) / HBAR
    t_start = (0.0 - x_src) / v
    line = CoupledGrid3(ctx, grid, wxy,
                        source=SheetSource(index=i_src, E0=g3["E0"], tau=g3["tau"], w0=w0, tpeak=0.0),
                        pol=1, waist=g3["waist"], gate=5e-9, t0=t_start)
    cache = args.tile_cache or os.path.join(tempfile.gettempdir(), "sbe_tiles.json")
    tiles = ctx.autotune(cache) if prec == _lib.PREC_MIXED else []
    # the beam in flight: Ey = E_inc(t - |x - x_src|/v) exp(-(y^2 + z^2)/waist^2),
    # Hz = sign(x - x_src) Ey(t - dt/2) / eta
    eta = np.sqrt(1.25663706127e-06 / (8.8541878188e-12 * MAT["epsr"]))
    prof = np.exp(-(y[:, None] ** 2 + z[None, :] ** 2) / g3["waist"] ** 2)

    def einc(t):
        return g3["E0"] * np.exp(-(t / g3["tau"]) ** 2) * np.cos(w0 * t)

    dist_x = np.abs(x - x_src)
    ex = einc(t_start - dist_x / v)
    hx = np.sign(x - x_src) * einc(t_start - dt / 2 - dist_x / v) / eta
    fe = 1.0 / (np.exp(np.minimum((ctx.table(0, "Ee").cpu().numpy() + MAT["gap"] / 2.0) /
                                  (1.380649e-23 * g3["temp"]), 700.0)) + 1.0)

    def fresh():
        E = torch.zeros((3,) + n, dtype=torch.complex128, device="cuda")
        H = torch.zeros_like(E)
        pr = torch.as_tensor(prof, device="cuda")
        E[1] = torch.as_tensor(ex, device="cuda")[:, None, None] * pr[None]
        H[2] = torch.as_tensor(hx, device="cuda")[:, None, None] * pr[None]
        dg = np.diag(fe).astype(complex)
        return ctx.zeros_state(), ctx.pack([dg] * nw), ctx.pack([dg] * nw), E, H

    st = fresh()
    line.reset()
    for _ in range(args.warmup):
        line.step(*st, dt, prec)
    torch.cuda.synchronize()
    ctx.profile(True)
    for cat in range(4):
        ctx.profile_read(cat)
    clk_dir = os.environ.get("SBE_CLOCKS_DIR", tempfile.gettempdir())
    clocks = ClockSampler(local, os.path.join(clk_dir, f"clocks_grid3_{rank}.csv"))
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record()
    torch.cuda.nvtx.range_push("timed_steps")   # ncu --nvtx-include timed_steps/
    for _ in range(args.steps):
        line.step(*st, dt, prec)
    torch.cuda.nvtx.range_pop()
    ev1.record()
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    clk = clocks.stop()
    prof_k = {cat: ctx.profile_read(cat) for cat in range(4)}
    ctx.profile(False)
    ctx.check()
    if dist:
        ms = max_over_ranks(dist, ms)
    value = job_rate(world, nw, args.steps, ms)
    graph = line.graph(*st, dt, prec)
    n_kernels = graph.kernels
    g0 = torch.cuda.Event(enable_timing=True)
    g1 = torch.cuda.Event(enable_timing=True)
    g0.record()
    for _ in range(args.steps):
        graph.launch()
    g1.record()
    torch.cuda.synchronize()
    graph_ms = g0.elapsed_time(g1) / args.steps
    graph.close()

    # end to end: the grid field E in from pinned host memory and the grid current J
    # back to pinned host memory every step (the wires' effect on the field)
    h_E = st[3].cpu().pin_memory()
    h_J = torch.empty((3,) + n, dtype=torch.complex128).pin_memory()
    Jv = line.view("J")
    torch.cuda.synchronize()
    e0e = torch.cuda.Event(enable_timing=True)
    e1e = torch.cuda.Event(enable_timing=True)
    e0e.record()
    for _ in range(args.steps):
        st[3].copy_(h_E, non_blocking=True)
        line.step(*st, dt, prec)
        h_J.copy_(Jv, non_blocking=True)
    e1e.record()
    torch.cuda.synchronize()
    e2e_ms = max_over_ranks(dist, e0e.elapsed_time(e1e))

    # the field step alone (H and E updates with the wires' current), its HBM roofline
    Et, Ht = st[3].clone(), st[4].clone()
    Jt = line.view("J").clone()
    for _ in range(3):
        grid.step(Et, Ht, Jt, dt)
    p0 = torch.cuda.Event(enable_timing=True)
    p1 = torch.cuda.Event(enable_timing=True)
    p0.record()
    for _ in range(20):
        grid.step(Et, Ht, Jt, dt)
    p1.record()
    torch.cuda.synchronize()
    field_ms = p0.elapsed_time(p1) / 20
    del Et, Ht, Jt

    # RHS error against FP64 at the current state and field on the wires
    P, C, D = st[0], st[1], st[2]
    Ek = line.view("Ek").clone()
    r64 = ctx.rhs(P, C, D, Ek, _lib.PREC_FP64)
    rmx = ctx.rhs(P, C, D, Ek, _lib.PREC_MIXED)
    rhs_err = max(float(torch.linalg.norm(a - b) / torch.linalg.norm(b)) for a, b in zip(rmx, r64))
    del r64, rmx

    fp64_ms = fp64_val = None
    if not args.no_fp64:
        st64 = tuple(t.clone() for t in st)
        torch.cuda.synchronize()
        f0 = torch.cuda.Event(enable_timing=True)
        f1 = torch.cuda.Event(enable_timing=True)
        f0.record()
        line.step(*st64, dt, _lib.PREC_FP64)
        f1.record()
        torch.cuda.synchronize()
        fp64_ms = max_over_ranks(dist, f0.elapsed_time(f1))
        fp64_val = job_rate(world, nw, 1, fp64_ms)
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    peaks, pk_kind = measured_peaks()
    N = n[0] * n[1] * n[2]
    field_bytes = N * (4 * 3 * 16 + 3 * 16)     # E, H read + write, J read (c128)
    hbm = peaks.get("hbm_gbs", 6800.0)
    achieved_gbs = field_bytes / (field_ms / 1e3) / 1e9
    comm_ms, comm_n = prof_k[0]
    per_eval_s = comm_ms / (4 * args.steps) / 1e3
    bf = peaks.get("bf16_tflops_sustained", 1700.0)
    line_out = {"metric": METRIC, "value": value, "unit": "wire-steps/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "fp16x3-f32acc/f64" if prec == _lib.PREC_MIXED else "f64",
                "data": "synthetic", "config": grid3_config(), "precision": args.precision,
                "clocks": clk,
                "e2e": {"value": job_rate(world, nw, args.steps, e2e_ms), "unit": "wire-steps/s",
                        "h2d_bytes_per_step": int(3 * N * 16), "d2h_bytes_per_step": int(3 * N * 16)},
                "gpu_launches": int(n_kernels * args.steps), "gpu_launches_per_step": int(n_kernels),
                "graph_replay_ms_per_step": graph_ms,
                # the dominant kernel of this workload is the commutator GEMM (64 wires of
                # Nk = 1024); the field step is reported beside it
                "roofline": {"bound": "tensor", "kernel": "k_tc_gemm (commutator dP/dC/dD)",
                             "achieved": 96.0 * nk ** 3 * nw / per_eval_s / 1e12, "peak": bf,
                             "unit": "TFLOP/s",
                             "frac": 96.0 * nk ** 3 * nw / per_eval_s / 1e12 / bf,
                             "peak_kind": f"{pk_kind} bf16 dense sustained",
                             "traffic": None, "ms_per_rhs_eval": per_eval_s * 1e3,
                             "launches": comm_n,
                             "flops_model": "algorithmic 96*Nk^3 per wire per RHS evaluation over "
                                            "the CUDA-event time of the evaluation's commutator "
                                            "launches"},
                "field_step": {"bound": "hbm",
                               "kernel": "3-D PSTD field step (plane transforms + curl + update)",
                               "achieved": achieved_gbs, "peak": hbm, "unit": "GB/s",
                               "frac": achieved_gbs / hbm, "peak_kind": f"{pk_kind} HBM copy",
                               "ms_per_field_step": field_ms,
                               "bytes_model": "E and H read and written, J read once: 240 B per "
                                              "grid point (c128), over the CUDA-event time of one "
                                              "step"},
                "step_tflops": 496.0 * nk ** 3 * nw * (args.steps / (ms / 1e3)) / 1e12,
                "tiles": tiles, "ctx_create_s": t_ctx,
                "fp64_gpu": {"value": fp64_val, "unit": "wire-steps/s", "ms_per_step": fp64_ms,
                             "steps": 1},
                "speedup_vs_fp64_gpu": (value / fp64_val) if fp64_val else None,
                "rhs_rel_err_vs_fp64": rhs_err,
                "cpu_baseline": None}
    print(json.dumps(line_out), flush=True)
    if dist:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--workload", default="multiwire", choices=sorted(WORKLOADS) + ["sweep", "grid3d"])
    ap.add_argument("--field-only", action="store_true",
                    help="grid3d: time the 3-D field step alone")
    ap.add_argument("--tile-cache", default=None,
                    help="JSON tile cache of the autotuner (default: in the temp directory)")
    ap.add_argument("--fp64-steps", type=int, default=3)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--ehs", action="store_true",
                    help="carrier-carrier scattering (EHs) on in every wire (not the default "
                         "workload's flags)")
    args = ap.parse_args()
    if args.ehs:
        FLAGS["EHs"] = True
    wl = WORKLOADS.get(args.workload)
    if args.impl == "reference":
        reference_arm(args, wl)
    elif args.workload == "grid3d":
        grid3_arm(args)
    elif wl is None:
        sweep_arm(args)
    else:
        gpu_arm(args, wl)


if __name__ == "__main__":
    main()
