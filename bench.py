"""Benchmark: batched mixed-precision SBE wire-steps/s on GB300.

Workload (default, "multiwire"): 32 identical GaAs-like quantum wires, Nk = 512
k points each (|k| <= 3e9 1/m, Nr = 1026), T = 300 K, Coulomb Hartree-Fock +
screening + LO-phonon relaxation + diagonal and off-diagonal dephasing, driven by
a Gaussian pulse E0 = 5e7 V/m, tau = 50 fs, hbar w0 = Eg + 20 meV, polarised
along the wires and retarded by the wire position (wires 100 nm apart), RK4 with
dt = 0.05 fs.  One step advances every wire by dt (4 RHS evaluations,
relaxation, charge normalisation and the polarisation/charge sources).

value     : wire-steps/s of the mixed path (tcgen05 FP16 hi/lo x3, FP32 accumulate,
            FP64 state) through WireContext.rk4_step with device-resident inputs.
e2e       : the same through the same call with the step's field copied from
            pinned host memory and the sources read back every step.
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
                      dt=0.05e-15, spacing=100e-9),
    # the same wires, fewer of them: the case the kernel-level profiles are taken on
    "profile": dict(nw=8, nk=512, kmax=3e9, temp=300.0, E0=5e7, tau=50e-15, det=20e-3,
                    dt=0.05e-15, spacing=100e-9),
}

MAT = dict(me=0.067 * ME0, mh=0.45 * ME0, gap=1.52 * E0C, HO=100e-3 * E0C, Delta0=6e-9,
           gam_e=1e12, gam_h=1e12, gam_eh=1e12, epsr=12.9, Oph=36e-3 * E0C / HBAR,
           Gph=3e-3 * E0C / HBAR)
FLAGS = dict(Optics=True, Excitons=True, EHs=False, Screened=True, Phonon=True, DCTrans=False,
             LF=True, FreePot=False, DiagDph=True, OffDiagDph=True, Recomb=False)
METRIC = "SBE wire-steps/s: batched mixed-prec vs plain FP64 GPU at ≤1e-6 rel err"


def wire_L(nk, kmax):
    return np.pi / (kmax / (nk / 2 - 0.5))


def pulse(t, wl):
    w0 = (MAT["gap"] + wl["det"] * E0C) / HBAR
    return wl["E0"] * np.exp(-t * t / wl["tau"] ** 2) * np.cos(w0 * t)


def wire_delays(wl):
    n = np.sqrt(MAT["epsr"])
    x = (np.arange(wl["nw"]) - (wl["nw"] - 1) / 2.0) * wl["spacing"]
    return x * n / C0


def env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


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


def reference_arm(args, wl):
    rank, world, local = env()
    if rank != 0:
        return
    times = cpu_wire_steps(wl, args.steps, args.warmup)
    tot = sum(times)
    v = len(times) / tot
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "wire-steps/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * tot / len(times), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config_of(wl, "reference"),
            "cpu_baseline": {"value": v, "unit": "wire-steps/s", "cores": os.cpu_count(),
                             "kind": "port",
                             "sample": f"one wire of the {wl['nw']}-wire batch, Nk={wl['nk']}, "
                                       f"{len(times)} RK4 steps (NumPy FP64 restatement; BLAS "
                                       "matmuls multi-threaded, O(Nk^3) sums single-threaded)"},
            "e2e": {"value": v, "unit": "wire-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def config_of(wl, impl):
    return {"workload": f"{wl['nw']} wires x Nk={wl['nk']} GaAs-like quantum wires, local "
                        f"retarded pulse E0={wl['E0']:.0e} V/m tau={wl['tau']*1e15:.0f} fs, "
                        f"T={wl['temp']:.0f} K, RK4 dt={wl['dt']*1e15:.2f} fs",
            "wires": wl["nw"], "nk": wl["nk"], "nr": 2 * wl["nk"] + 2,
            "flags": "Optics Excitons Screened Phonon LF DiagDph OffDiagDph",
            "integrator": "RK4 (coefficients frozen per step) + reference relaxation/normalisation",
            "l2": "inputs larger than L2 (FP64 state 403 MB, FP16 operand planes 1.9 GB per stage)",
            "impl": impl}


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
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.close()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in open(self.path):
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
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    ge.build()
    from pulsesuite_gb300 import _lib
    from pulsesuite_gb300.wires import WireContext, WireSpec

    nw, nk = wl["nw"], wl["nk"]
    L = wire_L(nk, wl["kmax"])
    specs = [WireSpec(nk=nk, L=L, temp=wl["temp"], wire_index=w + 1, flags=dict(FLAGS), **MAT)
             for w in range(nw)]
    ctx = WireContext(specs)
    prec = _lib.PREC_MIXED if args.precision == "mixed" else _lib.PREC_FP64
    nr = 2 * nk + 2
    wk = torch.stack([ctx.table(w, "window_k") for w in range(nw)])     # (nw, nr)
    delays = torch.as_tensor(wire_delays(wl), device="cuda")

    def field_k(t):
        """(nw, 3, nr) wire-k field of the retarded uniform pulse (along y)."""
        amp = torch.as_tensor(pulse(t - wire_delays(wl), wl), device="cuda")
        f = torch.zeros((nw, 3, nr), dtype=torch.complex128, device="cuda")
        f[:, 1, :] = amp[:, None] * wk
        return f

    fe = 1.0 / (np.exp((ctx.table(0, "Ee").cpu().numpy() + MAT["gap"] / 2.0) / 1.380649e-23
                       / wl["temp"]) + 1.0)

    def fresh_state():
        d = np.diag(fe).astype(complex)
        C = ctx.pack([d] * nw)
        D = ctx.pack([d] * nw)
        P = ctx.zeros_state()
        return P, C, D

    P, C, D = fresh_state()
    src = ctx.zeros_r(5)
    dt = wl["dt"]
    t = -2 * wl["tau"]
    Ek0 = torch.zeros(3 * ctx.total_r, dtype=torch.complex128, device="cuda")
    dEk = torch.zeros_like(Ek0)

    def set_field(t):
        f0 = field_k(t)
        f1 = field_k(t + dt)
        Ek0.copy_(f0.reshape(-1))
        dEk.copy_((f1 - f0).reshape(-1))

    # warm-up
    for _ in range(args.warmup):
        set_field(t)
        ctx.rk4_step(P, C, D, Ek0, dEk, dt, src, prec)
        t += dt
    torch.cuda.synchronize()

    # timed region: device-resident inputs, engine launches timed with events
    ctx.profile(True)
    for cat in range(4):
        ctx.profile_read(cat)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local, os.path.join(ROOT, "gpurun_out", f"clocks_{rank}.csv")) \
        if os.path.isdir(os.path.join(ROOT, "gpurun_out")) else ClockSampler(local, "/tmp/clk.csv")
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record()
    for _ in range(args.steps):
        set_field(t)
        ctx.rk4_step(P, C, D, Ek0, dEk, dt, src, prec)
        t += dt
    ev1.record()
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    clk = clocks.stop()
    if dist:
        tt = torch.tensor([ms], device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        ms = float(tt.item())
        dist.barrier()
    prof = {cat: ctx.profile_read(cat) for cat in range(4)}
    ctx.profile(False)
    value = world * nw * args.steps / (ms / 1e3)

    # CUDA graph of the same step (launch count, replay time)
    graph = ctx.rk4_graph(P, C, D, Ek0, dEk, dt, src, prec)
    n_kernels = graph.kernels
    set_field(t)
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

    # end to end: field from pinned host memory in, sources back to pinned host
    h_src = torch.empty(5 * ctx.total_r, dtype=torch.complex128).pin_memory()
    host_fields = []
    tt_ = t
    for _ in range(args.steps):
        f0 = field_k(tt_)
        f1 = field_k(tt_ + dt)
        host_fields.append((f0.reshape(-1).cpu().pin_memory(),
                            (f1 - f0).reshape(-1).cpu().pin_memory()))
        tt_ += dt
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for i in range(args.steps):
        Ek0.copy_(host_fields[i][0], non_blocking=True)
        dEk.copy_(host_fields[i][1], non_blocking=True)
        ctx.rk4_step(P, C, D, Ek0, dEk, dt, src, prec)
        h_src.copy_(src, non_blocking=True)
    e1.record()
    torch.cuda.synchronize()
    e2e_ms = e0.elapsed_time(e1)
    e2e_val = world * nw * args.steps / (e2e_ms / 1e3)

    # RHS error of the mixed path against the FP64 path at the current state
    Ek_now = field_k(t).reshape(-1).contiguous()
    r64 = ctx.rhs(P, C, D, Ek_now, _lib.PREC_FP64)
    rmx = ctx.rhs(P, C, D, Ek_now, _lib.PREC_MIXED)
    rhs_err = max(float(torch.linalg.norm(a - b) / torch.linalg.norm(b)) for a, b in zip(rmx, r64))

    # plain FP64 GPU path on the same state (a few steps: it is slow by design)
    fp64_ms = fp64_val = None
    n64 = max(1, args.fp64_steps)
    if not args.no_fp64:
        P2, C2, D2 = P.clone(), C.clone(), D.clone()
        set_field(t)
        ctx.rk4_step(P2, C2, D2, Ek0, dEk, dt, src, _lib.PREC_FP64)
        torch.cuda.synchronize()
        f0e = torch.cuda.Event(enable_timing=True)
        f1e = torch.cuda.Event(enable_timing=True)
        f0e.record()
        for _ in range(n64):
            ctx.rk4_step(P2, C2, D2, Ek0, dEk, dt, src, _lib.PREC_FP64)
        f1e.record()
        torch.cuda.synchronize()
        fp64_ms = f0e.elapsed_time(f1e) / n64
        fp64_val = world * nw / (fp64_ms / 1e3)

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return

    peaks, pk_kind = measured_peaks()
    comm_ms, comm_n = prof[0]
    per_launch_s = comm_ms / max(comm_n, 1) / 1e3
    useful = 32.0 * nk ** 3 * nw          # 4 complex terms x 8 flop x Nk^3 per wire
    executed = 96.0 * nk ** 3 * nw        # 12 FP16 MMA-GEMMs per term
    achieved = useful / per_launch_s / 1e12
    peak = peaks.get("bf16_tflops_sustained", 1700.0)
    roof = {"bound": "tensor", "kernel": "k_tc_gemm (commutator dP/dC/dD)", "achieved": achieved,
            "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
            "peak_kind": f"{pk_kind} bf16 dense sustained (fp16 dense has the same rate)",
            "executed_tflops": executed / per_launch_s / 1e12,
            "executed_frac": executed / per_launch_s / 1e12 / peak,
            "avg_launch_ms": per_launch_s * 1e3, "launches": comm_n,
            "traffic": None,
            "flops_model": "useful 32*Nk^3 per wire per launch (4 complex Nk^3 products); "
                           "executed 96*Nk^3 (4 real products x 3 hi/lo terms per complex term)"}
    other = {name: {"ms_per_step": prof[c][0] / args.steps, "launches": prof[c][1]}
             for c, name in ((1, "exchange_gemm"), (2, "source_gemm"), (3, "dephasing_fp32"))}

    cpu = None
    if not args.no_cpu:
        ct = cpu_wire_steps(wl, 1, 0)
        cpu = {"value": 1.0 / ct[0], "unit": "wire-steps/s", "cores": os.cpu_count(),
               "kind": "port",
               "sample": f"one RK4 wire-step of one wire (Nk={nk}) of this workload, NumPy FP64 "
                         "restatement (BLAS matmuls multi-threaded, O(Nk^3) sums single-threaded)"}

    line = {"metric": METRIC, "value": value, "unit": "wire-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "fp16x3-f32acc/f64" if prec == _lib.PREC_MIXED else "f64",
            "data": "synthetic", "config": config_of(wl, args.precision),
            "clocks": clk,
            "e2e": {"value": e2e_val, "unit": "wire-steps/s",
                    "h2d_bytes_per_step": int(2 * 3 * ctx.total_r * 16),
                    "d2h_bytes_per_step": int(5 * ctx.total_r * 16)},
            "gpu_launches": int(n_kernels * args.steps),
            "gpu_launches_per_step": int(n_kernels),
            "graph_replay_ms_per_step": graph_ms,
            "roofline": roof, "other_kernels": other,
            "fp64_gpu": {"value": fp64_val, "unit": "wire-steps/s", "ms_per_step": fp64_ms,
                         "steps": n64},
            "speedup_vs_fp64_gpu": (value / fp64_val) if fp64_val else None,
            "rhs_rel_err_vs_fp64": rhs_err,
            "cpu_baseline": cpu}
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--workload", default="multiwire", choices=sorted(WORKLOADS))
    ap.add_argument("--fp64-steps", type=int, default=2)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    args = ap.parse_args()
    wl = WORKLOADS[args.workload]
    if args.impl == "reference":
        reference_arm(args, wl)
    else:
        gpu_arm(args, wl)


if __name__ == "__main__":
    main()
