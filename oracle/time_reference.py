"""Time the reference's own SBE step on the host cores (test infrastructure).

Run from the repository root in a container that holds the reference source::

    python oracle/time_reference.py /path/to/pulsesuite/src oracle/reference_timing.json

The reference imports ``numba`` and ``pyfftw``; where they are not installed the two
stand-in packages of tests/golden/make_golden.py make ``numba.jit`` the identity (the
mode of the reference's own ``NUMBA_DISABLE_JIT=1`` target) and ``pyfftw`` NumPy's FFT.
The workload is the local-field wire of the task (one GaAs-like wire, Nk = 64, T = 77 K,
E0 = 1e6 V/m along y, tau = 100 fs, hbar w0 = Eg + 20 meV, dt = 0.1 fs from t = -2 tau)
through ``SBESolver`` + ``QWCalculator`` (its leapfrog step, one RHS evaluation per
step).  Writes the initialisation time, the seconds per step and the host description
as JSON (oracle/reference_timing.json); bench.py reports it inside its CPU-baseline
leg, labelled with the host it was measured on.
"""

import contextlib
import io
import json
import os
import platform
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "tests", "golden"))

import make_golden as MG  # noqa: E402

HBAR = 1.0545718176461565e-34
E0C = 1.602176634e-19
ME0 = 9.1093837139e-31


def cpu_model():
    try:
        with open("/proc/cpuinfo") as f:
            for ln in f:
                if ln.startswith("model name"):
                    return ln.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.processor() or platform.machine()


def main():
    src, out = sys.argv[1], sys.argv[2]
    nk, nsteps, warm = 64, 3, 1
    gap, me = 1.52 * E0C, 0.067 * ME0
    kmax = np.sqrt(1.2 * gap * 2.0 * me / HBAR ** 2)
    L = 32.5 * np.pi / kmax          # floor(kmax / (pi / L)) = 32: Nk = 64
    tau, E0, dt = 100e-15, 1e6, 0.1e-15
    w0 = (gap + 20e-3 * E0C) / HBAR
    with tempfile.TemporaryDirectory() as tmp:
        MG._install_stubs(tmp)
        sys.path.insert(0, tmp)
        sys.path.insert(1, os.path.abspath(src))
        run = os.path.join(tmp, "run")
        os.makedirs(os.path.join(run, "params"))
        cwd = os.getcwd()
        os.chdir(run)
        try:
            with open("params/qw.params", "w") as f:
                f.write(MG.QW_PARAMS.format(L=repr(float(L))))
            with open("params/mb.params", "w") as f:
                f.write(MG.MB_PARAMS)
            from pulsesuite.PSTD3D import SBEs
            nrr = 64
            rr = np.linspace(-1.25 * L, 1.25 * L, nrr)
            qrr = np.zeros(nrr)
            sink = io.StringIO()
            t0 = time.perf_counter()
            with contextlib.redirect_stdout(sink):
                s = SBEs.SBESolver(qrr, rr, 0.0, E0, 800e-9, 1, True)
            t_init = time.perf_counter() - t0
            assert s.Nk == nk, s.Nk
            times = []
            t = -2 * tau
            for n in range(warm + nsteps):
                e = E0 * np.exp(-t * t / tau ** 2) * np.cos(w0 * t)
                zeros = np.zeros(nrr, complex)
                Eyy = np.full(nrr, e, complex)
                outs = [np.zeros(nrr, complex) for _ in range(4)]
                a = time.perf_counter()
                with contextlib.redirect_stdout(sink):
                    s.QWCalculator(zeros, Eyy, zeros.copy(), zeros.copy(), rr, qrr, dt, 1, *outs,
                                   [True], [False])
                times.append(time.perf_counter() - a)
                t += dt
        finally:
            os.chdir(cwd)
    per = float(np.mean(times[warm:]))
    res = {"what": "reference SBESolver + QWCalculator (pure Python: numba absent, jit is the "
                   "identity; pyfftw as numpy.fft), leapfrog step, one RHS evaluation per step",
           "workload": "one GaAs-like wire, Nk=64, T=77 K, local field E0=1e6 V/m along y, "
                       "tau=100 fs, hbar w0=Eg+20 meV, dt=0.1 fs from t=-2 tau",
           "init_s": t_init, "s_per_step": per, "wire_steps_per_s": 1.0 / per,
           "steps_timed": nsteps, "warmup_steps": warm,
           "host": {"cpu": cpu_model(), "cpu_count": os.cpu_count(),
                    "machine": platform.machine(), "python": platform.python_version(),
                    "numpy": np.__version__}}
    with open(out, "w") as f:
        json.dump(res, f, indent=1)
    print(json.dumps(res))


if __name__ == "__main__":
    main()
