"""Benchmark of the semi-implicit spectral step at 256^3 (mixed vs FP64 GPU).

Workload: the 256x256x256 undulated-interface state (density ratio 0.8, Gaussian
psi noise sigma = 1e-3, seed 1002), reference coefficients, dt = 0.001 (the
reference's dt for 8 points per wavelength; dt = 0.01 diverges in the FP64 oracle
at step 20). A step is one full time step (loop body of smaiso-wcomp.cpp:1084-2198).

  value        mixed-path steps/s with the state resident in HBM (graph launches,
               CUDA events on the context's stream), normal-phase steps: the 50-step
               relax phase runs untimed first (its rate is reported on the side)
  e2e          the same metric through the C ABI with host buffers: swc_set_state
               from pinned host memory once, then per step swc_step_async(1) + the D2H
               read of that step's psi into pinned host memory
               (swc_get_field_async, overlapping the next step), all inside the
               timed region
  accuracy     both engines 2000 steps from the initial state: the mixed engine's
               psi / rho / mass / energy error against the FP64 engine
  roofline     the dominant kernel (the FP32 r2r axis pass, HBM-bound)
  cpu_baseline the FP64 CPU oracle on host cores (restatement of the reference loop,
               bit-identical to the reference's own code on the committed
               reference-run fixtures; the reference binary needs FFTW3-MPI and
               the MPI C++ bindings)

Multi-GPU: the path does not shard in this build (one GPU, no collectives); N
ranks run N independent replicas and value = N * steps / max-over-ranks time.
`--impl reference` times the CPU oracle port instead (rank 0 only).
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "steps/s at 256³: mixed vs FP64 GPU @ψ L2 err≤1e-5; gradient/forward time ratio"
N = 256
WORKLOAD = "undulated interface 256x256x256, density ratio 0.8, psi noise sigma 1e-3, dt 1e-3"
L2_BYTES = 129 * 2 ** 20


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--fp64-steps", type=int, default=None, help="timed FP64 steps (default: steps/5, >= 10)")
    ap.add_argument("--cpu-sample-steps", type=int, default=2)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--accuracy-steps", type=int, default=None,
                    help="run both engines this many steps from the initial state and report the mixed "
                         "engine's psi/rho/mass/energy error against the FP64 engine (0 skips it; default "
                         "the workload's run length: 2000 steps undulated, 1000 dislocations)")
    ap.add_argument("--grad-steps", type=int, default=40,
                    help="steps of the 128^3 FP64 adjoint timing (gradient/forward ratio); 0 skips it")
    ap.add_argument("--workload", choices=["undulated", "dislocations", "adjoint128", "adjoint256", "adjoint256_fp64"],
                    default="undulated",
                    help="dislocations: the 512x512x256 layer-dislocation configuration, reported as "
                         "its own JSON line (mixed and FP64 steps/s, mixed-vs-FP64 errors)")
    ap.add_argument("--adjoint-steps", type=int, default=None,
                    help="adjoint workloads: steps instead of the configuration's (short profiling runs)")
    ap.add_argument("--fd-mixed", action="store_true",
                    help="adjoint256: also 4th-order finite differences of the mixed forward (40 forward runs)")
    ap.add_argument("--energy-lambda", type=float, default=1.0,
                    help="adjoint workloads: weight of the free-energy diagnostic E(T) in the calibration loss")
    ap.add_argument("--divv-switch", type=int, default=None,
                    help="adjoint workloads and --only mixed/fp64: relax-phase length instead of the "
                         "reference's 50 (short profiling runs)")
    ap.add_argument("--only", choices=["mixed", "fp64", "pass"], default=None,
                    help="profiling mode: run only this engine's warm-up + timed steps and print its timing")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def make_params(precision, device=0):
    from smaiso_wcomp_gb300 import abi
    return abi.default_params(N, rho_0=0.8, divv_switch=50, precision=precision, device=device)


def initial_state(p):
    from smaiso_wcomp_gb300 import ic
    return ic.undulated_interface(p, seed=1002)


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def time_engine(p, psi, rho, warmup, steps, relax_steps=0):
    """Device-timed steps of one engine: CUDA events on the context's stream.

    The timed steps are normal-phase steps (the branch 97.5% of a 2000-step run takes):
    the relax phase (the reference's first divv_switch = 50 steps, REF:1312-1380) is
    run untimed first, then `warmup` untimed steps, then `steps` timed ones. With
    relax_steps > 0, that many relax-phase steps (after 3 untimed ones) are timed on the
    way and their ms/step returned as well."""
    from smaiso_wcomp_gb300.engine import Engine
    e = Engine(p)
    e.set_state(psi, rho)
    e.prepare()  # every step variant's graph (relax and normal phase) before the timed steps
    relax_ms = None
    if relax_steps > 0 and p.divv_switch >= relax_steps + 3:
        e.step(3)
        e.step(relax_steps)
        relax_ms = e.last_step_ms() / relax_steps
    if e.nloop < p.divv_switch:
        e.step(p.divv_switch - e.nloop)
    e.step(warmup)
    e.step(steps)
    ms = e.last_step_ms()
    launches = e.last_step_launches()
    return e, ms, launches, relax_ms


def time_e2e(p, psi_h, rho_h, steps):
    """Through the C ABI with host buffers: set_state from pinned host memory, then per
    step swc_step_async(1) and the D2H read of that step's psi into pinned host memory
    (swc_get_field_async into two alternating buffers: the copy of step n overlaps step
    n + 1), all inside the timed region, which ends when the last copy has landed and
    swc_sync has returned the steps' status. The value is the median of three timed
    runs of `steps` steps. The diagnostics run at the reference's cadence, every 50 steps
    (diag_interval). divv_switch = 0: every timed step takes the normal-phase branch, as
    the device-timed value's steps do (the relax phase would otherwise fill the first 50
    steps after swc_set_state, which the timed region has to include)."""
    from smaiso_wcomp_gb300 import abi
    from smaiso_wcomp_gb300.engine import Engine
    p = abi.SwcParams.from_buffer_copy(p)
    p.diag_interval = 50
    p.divv_switch = 0
    e = Engine(p)
    outs = [pinned((N, N, N)), pinned((N, N, N))]

    def run():
        e.set_state(psi_h, rho_h)
        for s in range(steps):
            e.step_async(1)
            e.field_async("psi", outs[s & 1])
        e.field_wait()
        e.sync()

    e.set_state(psi_h, rho_h)
    e.prepare()
    run()  # untimed: allocates the snapshots, warms the host-pinned copies
    times = []
    for _ in range(3):  # the median of three timed runs: host-side hiccups move single runs
        t0 = time.perf_counter()
        run()
        times.append(time.perf_counter() - t0)
    dt = float(np.median(times))
    e.close()
    h2d = 2 * psi_h.nbytes / steps
    return steps / dt, h2d, outs[0].nbytes


def pinned(shape):
    try:
        import torch
        if torch.cuda.is_available():
            return torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()
    except Exception:
        pass
    return np.empty(shape, dtype=np.float64)


def pass_roofline(precision, reps=5, fields=8):
    """Live CUDA-event timing of the dominant kernel -- one r2r axis pass over a 256^3
    field -- on the stream it is launched on, in the steady state of a step: `fields`
    distinct fields (8 x 67 MB FP32 = 537 MB, four times the 129 MB L2) each take a
    DCT-II axis pass, axis-major (all z passes, then all y, then all x), so every pass
    reads its field from DRAM and pays for the write-back of an earlier pass's output,
    as the passes of a step do; each axis's passes are replayed from a CUDA graph, as a
    step's are (the gaps between them included). Returns the mean time of one pass (ms),
    the per-axis means and the algorithmic bytes of one pass (one read + one write of
    the field)."""
    import torch
    from smaiso_wcomp_gb300 import abi
    from smaiso_wcomp_gb300.engine import R2RPlan
    dt = torch.float32 if precision == abi.SWC_PREC_MIXED else torch.float64
    if dt == torch.float64:
        fields = 4   # 4 x 134 MB, still four times L2
    xs = [torch.randn((N, N, N), dtype=dt, device="cuda") * 1e-3 for _ in range(fields)]
    plan = R2RPlan((N, N, N), (0, 0, 0), precision)
    s = torch.cuda.Stream()
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    per_axis = [[], [], []]
    # each axis's `fields` launches captured in one CUDA graph, as a step's passes are
    # (no host launch overhead between the passes)
    graphs = []
    for axis in (2, 1, 0):
        gr = torch.cuda.CUDAGraph()
        with torch.cuda.graph(gr, stream=s, capture_error_mode="relaxed"):
            for x in xs:
                plan.execute_axis(axis, x.data_ptr(), s.cuda_stream)
        graphs.append(gr)
    with torch.cuda.stream(s):
        for r in range(reps + 2):
            evs[0].record(s)
            for q, gr in enumerate(graphs):
                gr.replay()
                evs[q + 1].record(s)
            evs[3].synchronize()
            for x in xs:
                x.mul_(1.0 / (8 * N ** 3))   # keep the fields bounded (outside the timed region)
            if r >= 2:
                for q in range(3):
                    per_axis[q].append(evs[q].elapsed_time(evs[q + 1]) / fields)
    per_axis = [float(np.median(t)) for t in per_axis]
    elem = 4 if precision == abi.SWC_PREC_MIXED else 8
    alg_bytes = 2 * N ** 3 * elem
    del graphs, xs
    plan.close()
    return float(np.mean(per_axis)), per_axis, alg_bytes


def gradient_forward_ratio(steps, ckpt=20, n=128):
    """Wall time of swc_backward (segment recompute + adjoint steps) over the wall time
    of the forward steps it differentiates: FP64, n^3, checkpoints every `ckpt` steps."""
    import torch
    from smaiso_wcomp_gb300 import abi
    from smaiso_wcomp_gb300.engine import Engine
    p = abi.default_params(n, rho_0=0.8, divv_switch=min(50, steps // 2), adjoint_ckpt=ckpt)
    psi, rho = initial_state(p)
    e = Engine(p)
    e.set_state(psi, rho)           # warm-up: graph capture, adjoint buffers
    e.step(min(steps, ckpt))
    e.backward(dpsi=np.ones((n, n, n)))
    e.set_state(psi, rho)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e.step(steps)
    t1 = time.perf_counter()
    w = np.ones((n, n, n))
    g = e.backward(dpsi=w)
    t2 = time.perf_counter()
    e.close()
    return {"value": (t2 - t1) / (t1 - t0), "forward_s": t1 - t0, "backward_s": t2 - t1,
            "config": f"FP64 {n}^3, {steps} steps, checkpoint every {ckpt}, loss sum(psi(T))",
            "dL_dalpha": g["alpha"]}


CAL_COEFFS = ("alpha", "beta", "gamma", "nu", "rho_0")


def calibration_adjoint(which, steps=None, divv_switch=None, fd_mixed=False, lam=1.0):
    """The calibration-adjoint configurations: adjoint128 -- FP64 forward + FP64 adjoint,
    128^3, 400 steps, checkpoints every 20 steps; adjoint256 -- mixed forward + FP32
    adjoint, 256^3, 2000 steps, binomial checkpoint/recompute under a 40 GB device-memory
    cap (adjoint256_fp64: the same with the FP64 engine). Undulated
    interface, density ratio 0.8. psi_target comes from a run whose five coefficients are
    scaled by 1 + U(-0.1, 0.1) (seeded); loss L = ||psi(T) - psi_target||^2 + lam E(T),
    E(T) the free-energy diagnostic of the last step (REF:2214-2258; lam = 1 by default),
    differentiated by swc_backward_energy. Reports the gradient/forward wall-time ratio,
    the gradient and, for adjoint128, its error against central finite differences of the
    FP64 forward (h = 1e-6 relative, and 4th order). steps and divv_switch override the
    configuration's step count and relax-phase length (short profiling runs)."""
    from smaiso_wcomp_gb300 import abi, ic
    from smaiso_wcomp_gb300.engine import Engine
    n, nsteps = (128, 400) if which == "adjoint128" else (256, 2000)
    steps = steps or nsteps
    dv = {} if divv_switch is None else {"divv_switch": divv_switch}
    prec = abi.SWC_PREC_MIXED if which == "adjoint256" else abi.SWC_PREC_FP64
    mode = dict(adjoint_ckpt=20) if which == "adjoint128" else dict(adjoint_ckpt=-1, adjoint_cap_gb=40.0)
    mode["precision"] = prec
    base = abi.default_params(n, rho_0=0.8, **dv)
    psi0, rho0 = ic.undulated_interface(base)
    u = ic.uniform01(1004, np.arange(len(CAL_COEFFS), dtype=np.uint64))
    tgt = abi.default_params(n, rho_0=0.8, precision=prec, **dv)
    for c, x in zip(CAL_COEFFS, u):
        setattr(tgt, c, getattr(tgt, c) * (1.0 + 0.2 * (x - 0.5)))
    with Engine(tgt) as e:
        e.set_state(psi0, rho0)
        e.step(steps)
        psi_t = e.field("psi")

    def forward(q):
        with Engine(q) as e:
            e.set_state(psi0, rho0)
            e.step(steps)
            d = e.field("psi") - psi_t
            return float(np.sum(d * d)) + lam * e.diagnostics()["energy"]

    p = abi.default_params(n, rho_0=0.8, **mode, **dv)
    with Engine(p) as e:
        e.set_state(psi0, rho0)     # warm-up: graphs, adjoint buffers
        e.step(2)
        e.backward(dpsi=np.zeros((n, n, n)))
        e.set_state(psi0, rho0)
        t0 = time.perf_counter()
        e.step(steps)
        psi_T = e.field("psi")
        energy_T = e.diagnostics()["energy"]   # E(T): the diagnostics of the call's last step
        t1 = time.perf_counter()
        g = e.backward(dpsi=2.0 * (psi_T - psi_t), want_psi0=True, energy_lambda=lam)
        t2 = time.perf_counter()
    misfit = float(np.sum((psi_T - psi_t) ** 2))
    res = {"workload": f"calibration adjoint {n}^3, {steps} steps"
                       + ("" if divv_switch is None else f" (relax phase {divv_switch} steps)") + ", "
                       + ("mixed forward + FP32 adjoint, " if prec == abi.SWC_PREC_MIXED else
                          "FP64 forward + FP64 adjoint, ")
                       + ("checkpoints every 20 steps" if which == "adjoint128" else
                          "binomial checkpoint/recompute under a 40 GB cap"),
           "loss": {"lambda": lam, "misfit": misfit, "energy": energy_T, "total": misfit + lam * energy_T},
           "gradient_forward_ratio": (t2 - t1) / (t1 - t0), "forward_s": t1 - t0, "backward_s": t2 - t1,
           "forward_steps_rerun": g["forward_steps"], "snapshots": g["snapshots"],
           "adjoint_step_over_forward_step": ((t2 - t1) - g["forward_steps"] * (t1 - t0) / steps) / (t1 - t0),
           "gradient": {c: g[c] for c in CAL_COEFFS}}
    if which == "adjoint256" and fd_mixed:
        # 4th-order central differences of the mixed forward itself (the trajectory the
        # FP32 adjoint differentiates) at h = 1e-2 and 1e-3 relative: the forward's FP32
        # rounding makes L's noise too large for the h = 1e-6 of the FP64 check
        def at_m(c, x):
            q = abi.default_params(n, rho_0=0.8, precision=prec, **dv)
            setattr(q, c, x)
            return forward(q)
        for hr in (1e-2, 1e-3):
            fd4 = {}
            for c in CAL_COEFFS:
                v = getattr(p, c)
                h = hr * abs(v)
                fd4[c] = (8 * (at_m(c, v + h) - at_m(c, v - h)) - (at_m(c, v + 2 * h) - at_m(c, v - 2 * h))) / (12 * h)
            res[f"fd4_mixed_h{hr:g}"] = fd4
            res[f"rel_err_vs_fd4_mixed_h{hr:g}"] = {c: abs(g[c] - fd4[c]) / max(abs(fd4[c]), 1e-300)
                                                   for c in CAL_COEFFS}
    if which == "adjoint128":
        # central differences with the configuration's h = 1e-6 (relative), and 4th-order
        # central differences with h = 1e-3 (relative): at h = 1e-6 the FP64 roundoff of
        # L over 400 steps (~1e-13 |L|) divided by 2h dominates for the small gradients
        def at(c, x):
            q = abi.default_params(n, rho_0=0.8, **dv)
            setattr(q, c, x)
            return forward(q)
        fd, fd4 = {}, {}
        for c in CAL_COEFFS:
            v = getattr(p, c)
            h = 1e-6 * abs(v)
            fd[c] = (at(c, v + h) - at(c, v - h)) / (2 * h)
            h = 1e-3 * abs(v)
            fd4[c] = (8 * (at(c, v + h) - at(c, v - h)) - (at(c, v + 2 * h) - at(c, v - 2 * h))) / (12 * h)
        res["fd4_h1e-3"] = fd4
        res["rel_err_vs_fd4"] = {c: abs(g[c] - fd4[c]) / max(abs(fd4[c]), 1e-300) for c in CAL_COEFFS}
        d = ic.gaussian_noise((n, n, n), 77, 1.0)
        with Engine(abi.default_params(n, rho_0=0.8, **dv)) as e:
            def fpsi(x):
                e.set_state(psi0 + x * d, rho0)
                e.step(steps)
                r = e.field("psi") - psi_t
                return float(np.sum(r * r)) + lam * e.diagnostics()["energy"]
            fd_psi = (fpsi(1e-6) - fpsi(-1e-6)) / 2e-6
            # 4th-order differences at two steps: their truncation error falls as h^4,
            # their roundoff (~1e-13 |L| / h) grows as 1/h
            fd4s = {h: (8 * (fpsi(h) - fpsi(-h)) - (fpsi(2 * h) - fpsi(-2 * h))) / (12 * h) for h in (3e-5, 1e-5)}
            fd4_psi = fd4s[1e-5]
        res["fd"] = fd
        res["rel_err_vs_fd"] = {c: abs(g[c] - fd[c]) / max(abs(fd[c]), 1e-300) for c in CAL_COEFFS}
        ad_psi = float(np.sum(g["psi0"] * d))
        res["psi0_directional"] = {"adjoint": ad_psi, "fd": fd_psi, "rel_err": abs(ad_psi - fd_psi) / abs(fd_psi),
                                   "fd4_h3e-5": fd4s[3e-5], "fd4_h1e-5": fd4_psi,
                                   "rel_err_vs_fd4_h3e-5": abs(ad_psi - fd4s[3e-5]) / abs(fd4s[3e-5]),
                                   "rel_err_vs_fd4": abs(ad_psi - fd4_psi) / abs(fd4_psi)}
    return res


def accuracy_run(steps, device=0):
    """Both engines `steps` steps from the same state; relative L2 of psi and rho."""
    from smaiso_wcomp_gb300 import abi
    from smaiso_wcomp_gb300.engine import Engine
    out = {}
    psi, rho = initial_state(make_params(abi.SWC_PREC_MIXED, device))
    for prec in (abi.SWC_PREC_FP64, abi.SWC_PREC_MIXED):
        e = Engine(make_params(prec, device))
        e.set_state(psi, rho)
        e.step(steps)
        out[prec] = (e.field("psi"), e.field("rho"), e.diagnostics())
        e.close()
    rel = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))  # noqa: E731
    return {"steps": steps, "psi_rel_l2": rel(out[1][0], out[0][0]), "rho_rel_l2": rel(out[1][1], out[0][1]),
            "mass_rel": abs(out[1][2]["mass"] - out[0][2]["mass"]) / abs(out[0][2]["mass"]),
            "energy_rel": abs(out[1][2]["energy"] - out[0][2]["energy"]) / abs(out[0][2]["energy"])}


def dislocation_run(steps, warmup, acc_steps, device=0):
    """512x512x256 layer-dislocation workload (16 seeded edge-dislocation cores below a
    flat interface, density ratio 0.8): mixed and FP64 steps/s, and the mixed engine's
    psi / rho / v relative L2 error against the FP64 engine after acc_steps steps."""
    from smaiso_wcomp_gb300 import abi, ic
    from smaiso_wcomp_gb300.engine import Engine
    shape = (512, 512, 256)
    base = abi.default_params(*shape, rho_0=0.8)
    psi, rho = ic.dislocations(base)
    res = {"workload": "layer dislocations 512x512x256, 16 cores, density ratio 0.8, dt 1e-3",
           "points": int(np.prod(shape))}
    fields = {}
    for prec, name in ((abi.SWC_PREC_MIXED, "mixed"), (abi.SWC_PREC_FP64, "fp64")):
        p = abi.default_params(*shape, rho_0=0.8, precision=prec, device=device)
        with Engine(p) as e:
            e.set_state(psi, rho)
            e.step(acc_steps)
            fields[name] = {f: e.field(f) for f in ("psi", "rho", "vx", "vy", "vz")}
            n = steps if prec == abi.SWC_PREC_MIXED else max(5, steps // 10)
            e.step(warmup)
            e.step(n)   # graph-launched steps, CUDA events on the context's stream
            ms = e.last_step_ms() / n
        res[f"{name}_steps_per_s"] = 1e3 / ms
        res[f"{name}_ms_per_step"] = ms
    res["grid_point_steps_per_s"] = res["mixed_steps_per_s"] * res["points"]
    res["mixed_over_fp64"] = res["mixed_steps_per_s"] / res["fp64_steps_per_s"]
    a, b = fields["mixed"], fields["fp64"]
    rel = lambda x, y: float(np.linalg.norm(x - y) / np.linalg.norm(y))  # noqa: E731
    vn = np.sqrt(sum(np.linalg.norm(b[c]) ** 2 for c in ("vx", "vy", "vz")))
    dv = np.sqrt(sum(np.linalg.norm(a[c] - b[c]) ** 2 for c in ("vx", "vy", "vz")))
    res["errors_after_steps"] = acc_steps
    res["psi_rel_l2"], res["rho_rel_l2"], res["v_rel_l2"] = rel(a["psi"], b["psi"]), rel(a["rho"], b["rho"]), float(dv / vn)
    return res


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def cpu_baseline(steps, warmup=0):
    """FP64 CPU oracle on all host cores at the benchmark workload: `warmup` untimed and
    `steps` timed normal-phase steps (divv_switch = 0, so the sample's steps take the
    branch the GPU arm times; same state, same per-step work)."""
    from oracle import oracle as O
    from smaiso_wcomp_gb300 import abi
    cores = os.cpu_count() or 1
    O.set_threads(cores)
    p = make_params(abi.SWC_PREC_FP64)
    p.divv_switch = 0
    psi, rho = initial_state(p)
    o = O.Oracle(p)
    o.set_state(psi, rho)
    if warmup:
        o.step(warmup)
    t0 = time.perf_counter()
    o.step(steps)
    dt = time.perf_counter() - t0
    o.close()
    return {"value": steps / dt, "unit": "steps/s", "cores": cores, "kind": "port",
            "sample": f"{steps} timed FP64 oracle steps (after {warmup} untimed) of the 256^3 workload, "
                      f"normal phase, OpenMP {cores} threads (restatement of the reference loop, "
                      f"bit-identical to it on the reference-run fixtures)"}


# One oracle step of the 256^3 workload takes ~2.8 s on 16 Grace cores: the reference
# arm runs the declared warm-up and timed steps when they fit in REF_ARM_MAX_STEPS
# and otherwise the largest prefix that does, and prints the counts it ran.
REF_ARM_MAX_STEPS = 30


def config_of(world):
    return {"workload": WORKLOAD, "grid": [N, N, N], "parallelism": f"replicas{world}",
            "l2": f"inputs larger than L2 (working set {working_set_gb():.1f} GB > 129 MB L2)"}


def run_reference(args, rank):
    if rank != 0:
        return
    warmup = min(args.warmup, 3)
    steps = max(1, min(args.steps, REF_ARM_MAX_STEPS - warmup))
    base = cpu_baseline(steps, warmup)
    line = {"impl": "reference", "metric": METRIC, "value": base["value"], "unit": "steps/s",
            "n_gpus": args.gpus, "steps": steps, "warmup": warmup,
            "requested": {"steps": args.steps, "warmup": args.warmup},
            "ms_per_step": 1e3 / base["value"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config_of(args.gpus),
            "cpu_baseline": base,
            "e2e": {"value": base["value"], "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        return run_reference(args, rank)
    import torch
    torch.cuda.set_device(local)
    from smaiso_wcomp_gb300 import abi
    from smaiso_wcomp_gb300.engine import device_fma_peak
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
        pg = dist
    p_mix = make_params(abi.SWC_PREC_MIXED, device=local)
    psi, rho = initial_state(p_mix)
    if args.workload in ("adjoint128", "adjoint256", "adjoint256_fp64"):
        print(json.dumps(calibration_adjoint(args.workload, args.adjoint_steps, args.divv_switch, args.fd_mixed,
                                             args.energy_lambda)), flush=True)
        return
    if args.workload == "dislocations":
        acc_n = 1000 if args.accuracy_steps is None else (args.accuracy_steps or 50)
        print(json.dumps(dislocation_run(args.steps, args.warmup, acc_n, local)), flush=True)
        return
    if args.only == "pass":
        ms, per_axis, alg = pass_roofline(abi.SWC_PREC_MIXED, reps=args.steps)
        print(json.dumps({"only": "pass", "ms_per_pass": ms, "pass_ms_zyx": per_axis,
                          "gbs": alg / (ms * 1e-3) / 1e9}), flush=True)
        return
    if args.only:
        prec = abi.SWC_PREC_MIXED if args.only == "mixed" else abi.SWC_PREC_FP64
        po = make_params(prec, device=local)
        if args.divv_switch is not None:   # profiling runs: a shorter relax phase before the timed steps
            po.divv_switch = args.divv_switch
        e, ms, launches, _ = time_engine(po, psi, rho, args.warmup, args.steps)
        print(json.dumps({"only": args.only, "steps": args.steps, "ms_per_step": ms / args.steps,
                          "steps_per_s": args.steps / (ms * 1e-3), "gpu_launches": launches}), flush=True)
        e.close()
        return

    def barrier():
        torch.cuda.synchronize()
        if pg:
            pg.barrier()

    # mixed engine: the headline value (normal-phase steps; relax-phase rate on the side)
    barrier()
    with ClockSampler(local) as clk:
        e_mix, ms_mix, launches, relax_ms_mix = time_engine(p_mix, psi, rho, max(args.warmup, 3), args.steps,
                                                            relax_steps=20)
    barrier()
    clocks = clk.summary()
    e_mix.close()
    # FP64 engine on the same state, normal phase as well
    k64 = args.fp64_steps or max(10, args.steps // 5)
    p64 = make_params(abi.SWC_PREC_FP64, device=local)
    e_64, ms_64, _, relax_ms_64 = time_engine(p64, psi, rho, max(args.warmup, 3), k64, relax_steps=10)
    e_64.close()

    # max over ranks of the device time (replicas: no data-path collective)
    from smaiso_wcomp_gb300 import replicas
    ms_mix, ms_64 = replicas.max_over_ranks([ms_mix, ms_64], pg, device="cuda")
    sps_mix = replicas.job_throughput(args.steps, ms_mix * 1e-3, 1)
    sps_64 = replicas.job_throughput(k64, ms_64 * 1e-3, 1)
    # accuracy: both engines from the initial state through the relax phase and on
    # (spec bar: psi within 1e-5 of the FP64 engine after 2000 steps)
    if args.accuracy_steps is None:
        args.accuracy_steps = 2000
    acc = accuracy_run(args.accuracy_steps, local) if args.accuracy_steps > 0 else None

    psi_h = pinned((N, N, N))
    rho_h = pinned((N, N, N))
    psi_h[...] = psi
    rho_h[...] = rho
    e2e_sps, h2d, d2h = time_e2e(p_mix, psi_h, rho_h, max(10, args.steps))

    peaks, peak_kind = load_peaks()
    ms_pass, axes_ms, alg = pass_roofline(abi.SWC_PREC_MIXED)
    achieved = alg / (ms_pass * 1e-3) / 1e9
    ms_pass64, axes64_ms, alg64 = pass_roofline(abi.SWC_PREC_FP64)
    fp64_peak = device_fma_peak(abi.SWC_PREC_FP64)
    # algorithmic flops of one r2r axis pass: (2.5 log2 n + 8) n per line of length n
    # (real-data FFT plus the DCT pre/post twiddles), n^2 lines
    fp64_flops = (2.5 * np.log2(N) + 8.0) * N ** 3
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": achieved / peaks["hbm_gbs"], "traffic": PASS_TRAFFIC.get("fp32"),
                "kernel": "r2r_tma_kernel<256, C2> (one FP32 DCT-II axis pass, 256^3, steady state of 8 fields, mean of z/y/x)",
                "pass_ms_zyx": axes_ms, "alg_bytes_per_launch": alg,
                "peak_source": f"{peak_kind} hbm_gbs"}
    line = {
        "metric": METRIC, "value": sps_mix * world, "unit": "steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_mix / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": config_of(world),
        "phase": "normal (steps after the 50-step relax phase)",
        "relax_phase_steps_per_s": 1e3 / relax_ms_mix if relax_ms_mix else None,
        "fp64_steps_per_s": sps_64 * world, "mixed_over_fp64": sps_mix / sps_64,
        "fp64_relax_phase_steps_per_s": 1e3 / relax_ms_64 if relax_ms_64 else None,
        "grid_point_steps_per_s": sps_mix * world * N ** 3,
        "psi_rel_l2_mixed_vs_fp64": acc["psi_rel_l2"] if acc else None,
        "rho_rel_l2_mixed_vs_fp64": acc["rho_rel_l2"] if acc else None,
        "accuracy_steps": acc["steps"] if acc else 0,
        "accuracy": acc,
        "gradient_forward_ratio": None,  # filled below
        "e2e": {"value": e2e_sps * world, "unit": "steps/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "roofline": roofline,
        "roofline_fp64_pass": {"bound": "fp64_alu", "achieved": fp64_flops / (ms_pass64 * 1e-3) / 1e12,
                               "peak": fp64_peak, "unit": "TFLOP/s",
                               "frac": fp64_flops / (ms_pass64 * 1e-3) / 1e12 / fp64_peak,
                               "hbm_gbs": alg64 / (ms_pass64 * 1e-3) / 1e9,
                               "peak_source": "measured swc_device_fma_peak(FP64)"},
        "gpu_launches": launches,
        "clocks": clocks,
    }
    if args.grad_steps > 0:
        gr = gradient_forward_ratio(args.grad_steps)
        line["gradient_forward_ratio"] = gr["value"]
        line["gradient"] = gr
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args.cpu_sample_steps)
        # matched precision: the FP64 GPU engine over the FP64 CPU oracle
        line["fp64_gpu_over_cpu"] = sps_64 / line["cpu_baseline"]["value"]
        line["mixed_gpu_over_cpu"] = sps_mix / line["cpu_baseline"]["value"]
    if rank == 0:
        print(json.dumps(line), flush=True)
    if pg:
        pg.destroy_process_group()


# DRAM bytes (read + write) per launch of the dominant kernel in the steady state that
# pass_roofline times (mean of its z/y/x passes), from the ncu capture with
# --cache-control none summarised in profiles/r2r_tma_fp32_n256_256cubed.md.
PASS_TRAFFIC = {"fp32": 132.3e6}


def working_set_gb():
    return (38 * 4 + 4 * 8) * N ** 3 / 1e9


if __name__ == "__main__":
    main()
