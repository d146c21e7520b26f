"""Benchmark of the GB300 MHD + KI cooling step (one JSON line on rank 0).

Workload: the 256^3 colliding warm-neutral-medium flows with KI cooling
(20 pc box, n0 = 1 cm^-3, T0 = 6000 K, lognormal density rms 0.1 with a
k^-11/3 spectrum from ran0 seed 1, vx = +-20 km/s converging at the
mid-plane, |B| = 3 uG at 45 deg in x-y, free x and periodic y/z
boundaries, DISSIP on).  A "step" is one EVOLVE iteration: dt from
Couran+Stblty, SOURCE(dt/2), three sweeps, constrained transport,
SOURCE(dt/2), DISSIP.  The resident grid (28 FP64 arrays of 260^3, state
plus scratch, 3.9 GB, and 15 FP32 scratch arrays, 1.05 GB) is far larger
than the 129 MB L2, so no flush is needed between steps.

`value` is the chosen form (FP32 reconstruction/flux, FP64 accumulation);
`plain_fp64` is the plain FP64 path timed the same way; `l1_error` compares
the two at the same physical time after --l1-steps FP64 steps (each form
takes its own dt).  `e2e` times the same step
through the C ABI entry mhd_step_host: every step copies the whole state in
from pinned host memory and the new state out, the finished arrays (rho and
species after the sweeps, the face field after CT) while the step still
runs; its value is the median of 12 individually timed steps (the mean and
the samples are in the line too).  `roofline` is for the dominant kernel (the
fused sweep), with algorithmic bytes from the per-zone budget of the step.
`cpu_baseline` is the CPU restatement (oracle, C++ with OpenMP) timed on a
bounded sample on the host cores.  `stiff_cooling_source` times SOURCE alone
in the stiff regime of the KI cooling (30x density, dt = 0.05), where the
surrogate replaces the implicit bisection: FP64, FP32 exact and FP32 +
surrogate from the same state, with the pressure error against FP64.

`config2` is the 128^3 decaying Mach-5 MHD turbulence (periodic, plain FP64,
100 steps at CFL 0.4) with its mass / momentum drift and max |div B|, and the
chosen form beside it; `config5` is the 512^3 colliding flow (10 pc
perturbation scale) in the chosen form with the trained surrogate, 100
steps, with event times and HBM roofline fractions per phase of the step,
next to the plain FP64 path at the same size.

`--impl reference` times that CPU restatement alone (the reference itself is
Fortran + MPI and no Fortran compiler exists on this machine; the restatement
reproduces its golden outputs) on the same 256^3 problem: --warmup untimed
and --steps timed full steps.
"""
import argparse
import json
import os
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

B_ALG_STEP = 552.0      # algorithmic bytes per zone-update of the whole step
B_ALG_SWEEP = 104.0     # per sweep: read rho, v3, p, face-B3 (64) + write rho, v3, p (40)
# algorithmic bytes per zone of each phase of the step (they add up to B_ALG_STEP)
B_ALG_PHASE = {"timestep": 64.0, "source_1": 48.0, "sweep_x": 104.0, "sweep_y": 104.0, "sweep_z": 104.0,
               "ct": 80.0, "source_2": 48.0, "dissip": 0.0,
               # self-gravity (not part of the 552 B/zone step): read rho, write Phi; read Phi, v + write v
               "gravity_potential": 16.0, "gravity_kick_1": 56.0, "gravity_kick_2": 56.0}
SWEEP_NAMES = ("sweep_x", "sweep_y", "sweep_z")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-stiff", action="store_true", help="skip the stiff-cooling SOURCE comparison")
    ap.add_argument("--l1-steps", type=int, default=100,
                    help="FP64 steps of the accuracy comparison (the chosen form runs to the same time)")
    ap.add_argument("--no-config2", action="store_true", help="skip the 128^3 turbulence sub-run")
    ap.add_argument("--no-config5", action="store_true", help="skip the 512^3 sub-run")
    ap.add_argument("--no-gravity", action="store_true", help="skip the self-gravity timing")
    ap.add_argument("--stiff-only", action="store_true",
                    help="train the surrogate and run only the stiff-cooling comparison (prints that object)")
    ap.add_argument("--sur-steps", type=int, default=2000)
    ap.add_argument("--sur-data", type=int, default=1 << 24)
    return ap.parse_args()


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profile_value(fname, key):
    """A `key=value` figure from a committed ncu summary under profiles/."""
    path = os.path.join(ROOT, "profiles", fname)
    try:
        for line in open(path):
            if line.startswith(key + "="):
                return float(line.split("=")[1])
    except OSError:
        pass
    return None


def ncu_traffic():
    """DRAM bytes per zone of one sweep launch from the committed ncu summary."""
    return profile_value("sweep_fp32_traffic.txt", "dram_bytes_per_zone_fp32_sweep")


class ClockSampler:
    """nvidia-smi clocks during the timed region (one sample every 50 ms).

    The sampler is started first and the region begins once nvidia-smi has
    produced its first line; only lines read between __enter__'s return and
    __exit__ are kept."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []
        self._all = []
        self._t0 = self._t1 = None

    def _reader(self):
        for line in self.proc.stdout:
            if line.strip():
                self._all.append((time.perf_counter(), line))

    def __enter__(self):
        import threading
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        if self.proc:
            threading.Thread(target=self._reader, daemon=True).start()
            deadline = time.perf_counter() + 5.0
            while not self._all and time.perf_counter() < deadline and self.proc.poll() is None:
                time.sleep(0.01)
        self._t0 = time.perf_counter()
        return self

    def __exit__(self, *a):
        self._t1 = time.perf_counter()
        if self.proc:
            time.sleep(0.06)   # the sample that covers the end of the region
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.proc.wait()
            self.lines = [l for t, l in self._all if self._t0 <= t <= self._t1 + 0.06]

    def summary(self):
        import statistics
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            f = [x.strip() for x in l.split(",")]
            try:
                sm.append(float(f[0]))
                mx = float(f[1])
            except (ValueError, IndexError):
                continue
            for n, v in zip(names, f[3:7]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(n=256, steps=2):
    """The oracle (C++ restatement, OpenMP over host cores) on the same
    256^3 problem, a bounded sample of 2 full steps after one untimed step:
    zone-updates/s."""
    from code_tohoku_gb300 import problems
    from oracle.pyoracle import Oracle3D
    st = problems.colliding_flows(n)
    o = Oracle3D(st.params)
    o.upload(st)
    o.step()   # first-touch and thread start-up
    t = time.perf_counter()
    for _ in range(steps):
        o.step()
    el = time.perf_counter() - t
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    return {"value": n ** 3 * steps / el, "unit": "zone-updates/s", "cores": cores, "kind": "port",
            "sample": f"{steps} full steps of the {n}^3 colliding-flow problem (the headline workload), "
                      "after one untimed step"}


def run_reference(args, rank):
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    from code_tohoku_gb300 import problems
    from oracle.pyoracle import Oracle3D
    n = args.n
    st = problems.colliding_flows(n)
    o = Oracle3D(st.params)
    o.upload(st)
    for _ in range(max(args.warmup, 0)):
        o.step()
    t = time.perf_counter()
    for _ in range(args.steps):
        o.step()
    el = time.perf_counter() - t
    v = n ** 3 * args.steps / el
    line = {"metric": "zone-updates/s, 256^3 MHD+KI cool: FP32+surrogate vs plain FP64 at stated L1 err",
            "value": v, "unit": "zone-updates/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": f"colliding WNM flows with KI cooling, {n}^3, free x / periodic y,z",
                       "n": n, "precision": "fp64"},
            "cpu_baseline": {"value": v, "unit": "zone-updates/s", "cores": int(os.environ["OMP_NUM_THREADS"]),
                             "kind": "port",
                             "sample": f"{args.steps} full steps of the {n}^3 problem after {args.warmup} "
                                       "untimed ones; C++ restatement of MCF3DSGincfca3.f90 (no Fortran "
                                       "compiler on this machine)"},
            "e2e": {"value": v, "unit": "zone-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    rank, world, local = dist_info()
    if args.impl == "reference":
        run_reference(args, rank)
        return
    import numpy as np
    import torch

    from code_tohoku_gb300 import native, problems, replicas
    torch.cuda.set_device(local)
    replicas.init("nccl")
    dev = local
    # a dedicated stream: the kernels, the CUDA events and the copies all go here
    stream = torch.cuda.Stream()

    st = problems.colliding_flows(args.n)
    n3 = args.n ** 3

    # the learned part: train the KI-cooling surrogate on this GPU first
    from code_tohoku_gb300 import surrogate
    t0 = time.perf_counter()
    sur_params, hist = surrogate.train(n_data=args.sur_data, batch=65536, steps=args.sur_steps, lr=1e-3,
                                       seed=1, device=dev)
    sur_train_s = time.perf_counter() - t0

    def make(prec, cooling=native.COOL_EXACT, state=None):
        state = st if state is None else state
        g = native.Mhd3D(state.params, precision=prec, cooling=cooling, device=dev)
        g.set_stream(stream.cuda_stream)
        if cooling == native.COOL_SURROGATE:
            g.surrogate_load(sur_params, 1e-3)
        g.upload(state)
        return g

    def barrier():
        replicas.barrier()
        torch.cuda.synchronize()

    def step_timed(g, rec, dissip):
        """One EVOLVE iteration through the C ABI (the calls mhd_step makes),
        with CUDA events on the handle's stream around every phase when rec
        (phase -> list of event pairs) is given."""
        def phase(name, fn, *a):
            if rec is None:
                return fn(*a)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            r = fn(*a)
            e1.record(stream)
            rec.setdefault(name, []).append((e0, e1))
            return r
        dt, _ = phase("timestep", g.timestep)
        grav = getattr(g.params, "ifgrv", 0) == 2
        if grav:
            phase("gravity_kick_1", g.gravity, dt, 3)            # EVOLVE :607
        phase("source_1", g.source, 0.5 * dt)
        order = ((0, 1, 2), (1, 2, 0), (2, 0, 1), (0, 2, 1), (1, 0, 2), (2, 1, 0))[g.ifevo - 1]
        for d in order:
            phase(SWEEP_NAMES[d], g.sweep, d, dt)
        g.ifevo = g.ifevo % 6 + 1
        phase("ct", g.ct, dt)
        phase("source_2", g.source, 0.5 * dt)
        if grav:
            phase("gravity_potential", g.gravity, dt, 2)         # :653
            phase("gravity_kick_2", g.gravity, dt, 3)
        if dissip:
            phase("dissip", g.dissip)
        g.set_time(g.time + dt, g.ifevo)
        return dt

    def phase_ms(rec):
        return {k: sum(a.elapsed_time(b) for a, b in v) / len(v) for k, v in rec.items()}

    def phase_roofline(pms, n3, hbm):
        """Per phase: mean event time, algorithmic bytes / time, fraction of HBM."""
        out = {}
        for k, ms in pms.items():
            gbs = B_ALG_PHASE[k] * n3 / (ms * 1e-3) / 1e9 if B_ALG_PHASE[k] else None
            out[k] = {"ms": ms, "alg_bytes_per_zone": B_ALG_PHASE[k], "achieved_gbs": gbs,
                      "frac_of_measured_hbm": gbs / hbm if gbs else None}
        return out

    def timed_run(prec, cooling=native.COOL_EXACT, state=None, steps=None, warmup=None, fresh=False):
        """Warm-up steps, then `steps` timed steps; fresh: upload the initial
        state again after the warm-up, so the timed steps are steps 1..steps
        of the run."""
        state = st if state is None else state
        steps = args.steps if steps is None else steps
        warmup = args.warmup if warmup is None else warmup
        g = make(prec, cooling, state)
        g.diag0 = g.diagnostics()
        g.ifevo = 1
        for _ in range(warmup):
            step_timed(g, None, state.params.dissip)
        if fresh:
            g.upload(state)
            g.set_time(0.0, 1)
            g.ifevo = 1
        rec = {}
        barrier()
        launches0 = g.kernel_launches
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        with ClockSampler(dev) as clk:
            e0.record(stream)
            for _ in range(steps):
                step_timed(g, rec, state.params.dissip)
            e1.record(stream)
            barrier()
        ms = e0.elapsed_time(e1)
        launches = g.kernel_launches - launches0
        return g, ms, phase_ms(rec), launches, clk.summary()

    def divb_split(g_, state):
        """max |div B| over the interior cells, and over those not next to a
        free x boundary (there the reference's face exchange rewrites face
        n+1, so the last cell's div B is not round-off)."""
        U_ = g_.download(with_bcc=False)[0]
        n_ = state.params.nx
        c = slice(2, 2 + n_)
        d = ((U_[5][c, c, 3:3 + n_] - U_[5][c, c, 2:2 + n_]) / state.dx[2:2 + n_][None, None, :]
             + (U_[6][c, 3:3 + n_, c] - U_[6][c, 2:2 + n_, c]) / state.dy[2:2 + n_][None, :, None]
             + (U_[7][3:3 + n_, c, c] - U_[7][2:2 + n_, c, c]) / state.dz[2:2 + n_][:, None, None])
        a = np.abs(d)
        lo = 1 if state.params.bc[0] == 1 else 0
        hi = n_ - 1 if state.params.bc[1] == 1 else n_
        return float(a.max()), float(a[:, :, lo:hi].max())

    def stiff_comparison():
        # The stiff regime of KI cooling, where the learned part works: the same
        # colliding flow at 30x the density (n = 30 cm^-3) and SOURCE(dt) with
        # dt = 0.05 Myr, longer than the cooling time of most cells.  SOURCE only,
        # from the same uploaded state each time; the FP64 form gives the
        # reference pressure.
        sst = problems.colliding_flows(args.n)
        sst.U[0] *= 30.0
        sst.species *= 30.0
        sdt = 0.05
        stiff = {"state": "colliding flow at 30x density", "dt": sdt}
        p_ref = None
        for name, prec, cool in (("fp64", native.PREC_FP64, native.COOL_EXACT),
                                 ("fp32_exact", native.PREC_FP32, native.COOL_EXACT),
                                 ("fp32_surrogate", native.PREC_FP32, native.COOL_SURROGATE),
                                 ("fp32_newton_no_network", native.PREC_FP32, native.COOL_NEWTON)):
            gs = native.Mhd3D(sst.params, precision=prec, cooling=cool, device=dev)
            gs.set_stream(stream.cuda_stream)
            if cool == native.COOL_SURROGATE:
                gs.surrogate_load(sur_params, 1e-3)
            times = []
            for _ in range(3):
                gs.upload(sst)
                gs.reset_counters()
                barrier()
                a = torch.cuda.Event(enable_timing=True)
                b = torch.cuda.Event(enable_timing=True)
                a.record(stream)
                gs.source(sdt)
                b.record(stream)
                barrier()
                times.append(a.elapsed_time(b))
            d = gs.diagnostics()
            pp = gs.download(with_bcc=False)[0][4][2:-2, 2:-2, 2:-2]
            if p_ref is None:
                p_ref = pp
            stiff[name] = {"ms_per_source": min(times), "bisection_cells": d["imc_cells"],
                           "guess_accepted_cells": d["surrogate_cells"], "guess_rejected_cells": d["fallback_cells"],
                           "l1_p_vs_fp64": float(np.abs(pp - p_ref).mean() / np.abs(p_ref).mean())}
            del gs
        stiff["surrogate_speedup_vs_fp32_exact"] = (stiff["fp32_exact"]["ms_per_source"] /
                                                    stiff["fp32_surrogate"]["ms_per_source"])
        stiff["surrogate_speedup_vs_newton_no_network"] = (stiff["fp32_newton_no_network"]["ms_per_source"] /
                                                           stiff["fp32_surrogate"]["ms_per_source"])
        for k in ("fp32_surrogate", "fp32_newton_no_network"):
            r = stiff[k]
            r["fallback_fraction"] = r["guess_rejected_cells"] / max(1, r["guess_rejected_cells"] + r["guess_accepted_cells"])

        # The same solvers inside whole steps: the colliding flow at 3000x the
        # density (n = 3000 cm^-3 at 6000 K cools in ~4e-4 Myr), where the
        # reference's own time-step control leaves the cells stiff (the
        # cooling-time limit 0.2 t_cool is floored at 2.5e-4 Myr, Stblty
        # :2806).  At 30x the step's dt follows 0.2 t_cool and no cell is
        # stiff; hence this density.  Steps 1..K from the uploaded state, each
        # event-timed; FP64 runs the same steps for the error.
        kst = 4
        wst = problems.colliding_flows(args.n)
        wst.U[0] *= 3000.0
        wst.species *= 3000.0
        wst.U[4] *= 3000.0          # the same 6000 K
        steps_stiff = {"state": "colliding flow at 3000x density, 6000 K", "steps": kst}
        u_ref = None
        for name, prec, cool in (("fp64", native.PREC_FP64, native.COOL_EXACT),
                                 ("fp32_exact", native.PREC_FP32, native.COOL_EXACT),
                                 ("fp32_surrogate", native.PREC_FP32, native.COOL_SURROGATE),
                                 ("fp32_newton_no_network", native.PREC_FP32, native.COOL_NEWTON)):
            gs = native.Mhd3D(wst.params, precision=prec, cooling=cool, device=dev)
            gs.set_stream(stream.cuda_stream)
            if cool == native.COOL_SURROGATE:
                gs.surrogate_load(sur_params, 1e-3)
            gs.upload(wst)
            gs.reset_counters()
            rec = {}
            barrier()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            dts = []
            gs.ifevo = 1
            for _ in range(kst):
                dts.append(step_timed(gs, rec, wst.params.dissip))
            e1.record(stream)
            barrier()
            d = gs.diagnostics()
            U = gs.download(with_bcc=False)[0]
            c = (slice(2, -2),) * 3
            if u_ref is None:
                u_ref = (U[0][c].copy(), U[4][c].copy())
            steps_stiff[name] = {"ms_per_step": e0.elapsed_time(e1) / kst, "phase_ms": phase_ms(rec), "dt": dts,
                                 "bisection_cells": d["imc_cells"], "guess_accepted_cells": d["surrogate_cells"],
                                 "guess_rejected_cells": d["fallback_cells"],
                                 "l1_rho_vs_fp64": float(np.abs(U[0][c] - u_ref[0]).mean() / np.abs(u_ref[0]).mean()),
                                 "l1_p_vs_fp64": float(np.abs(U[4][c] - u_ref[1]).mean() / np.abs(u_ref[1]).mean())}
            del gs
        steps_stiff["surrogate_speedup_vs_fp32_exact"] = (steps_stiff["fp32_exact"]["ms_per_step"] /
                                                          steps_stiff["fp32_surrogate"]["ms_per_step"])
        stiff["whole_steps"] = steps_stiff
        return stiff

    hbm, which = peaks()
    if args.stiff_only:
        stiff = stiff_comparison()
        if rank == 0:
            print(json.dumps({"stiff_cooling_source": stiff, "n": args.n}), flush=True)
        return
    # chosen form: FP32 reconstruction/flux + FP64 accumulation + surrogate
    g32, ms32, ph32, launches32, clocks = timed_run(native.PREC_FP32, native.COOL_SURROGATE)
    d32 = g32.diagnostics()
    divb256 = divb_split(g32, st)
    sw32 = [ph32[k] for k in SWEEP_NAMES]
    ms32 = replicas.max_over_ranks(ms32)
    value = world * n3 * args.steps / (ms32 * 1e-3)
    # ablation: the same FP32 form with the exact cooling integrator
    gx, msx, _, _, _ = timed_run(native.PREC_FP32, native.COOL_EXACT)
    dx_ = gx.diagnostics()
    del gx

    # the FP64 pipe of this GPU, measured: the plain form's roofline
    fp64_peak = native.fp64_peak(dev)

    # plain FP64 form, same workload
    fp64 = None
    l1 = None
    if not args.no_fp64:
        g64, ms64, ph64, launches64, _ = timed_run(native.PREC_FP64)
        sweep64 = sum(ph64[k] for k in SWEEP_NAMES) / 3
        fp64 = {"value": n3 * args.steps / (ms64 * 1e-3), "unit": "zone-updates/s",
                "ms_per_step": ms64 / args.steps, "sweep_ms": sweep64, "phase_ms": ph64}
        # FP64 operations per zone of one plain sweep launch (ncu instruction
        # counts: 2 per DFMA, 1 per DADD / DMUL), against the measured FMA rate
        fl = profile_value("sweep_fp64_pipe.txt", "fp64_flops_per_zone_fp64_sweep")
        pipe = profile_value("sweep_fp64_pipe.txt", "fp64_pipe_active_pct")
        if fl:
            ach = fl * n3 / (sweep64 * 1e-3) / 1e9
            fp64["roofline"] = {"bound": "fp64 pipe", "kernel": "sweep_kernel<DIR, P, double>",
                                "achieved": ach, "peak": fp64_peak["fma_gflops"], "unit": "GFLOP/s",
                                "frac": ach / fp64_peak["fma_gflops"], "flops_per_zone": fl,
                                "peak_source": "mhd_fp64_peak (measured in this run: dependent FMA chains)",
                                "ncu_fp64_pipe_active_pct": pipe}
        # L1 error of the chosen form against FP64 at the same physical time:
        # FP64 runs --l1-steps steps in all, the chosen form runs to that
        # time (each form takes its own dt, like a run; the last step of the
        # chosen form is clipped to land on it)
        done = args.warmup + args.steps
        if args.l1_steps > done:
            g64.evolve(args.l1_steps - done)
        t64 = g64.time
        g32.reset_counters()
        g32.evolve(2 * args.l1_steps + 10, tsave=t64)
        d_acc = g32.diagnostics()
        U32, s32, b32 = g32.download()
        U64, s64, b64 = g64.download()
        c = (slice(2, -2),) * 3

        def l1rel(a, b):
            return float(np.abs(a - b).mean() / np.abs(b).mean())
        n32 = s32[0][c] + s32[1][c] + s32[2][c] + s32[3][c] + s32[4][c]
        n64 = s64[0][c] + s64[1][c] + s64[2][c] + s64[3][c] + s64[4][c]
        l1 = {"rho": l1rel(U32[0][c], U64[0][c]), "T": l1rel(U32[4][c] / n32, U64[4][c] / n64),
              "B": l1rel(b32[(slice(None),) + c], b64[(slice(None),) + c]),
              "steps_fp64": max(args.l1_steps, args.warmup + args.steps), "time": t64,
              "time_fp32": g32.time,
              "cooling_cells": {"surrogate": d_acc["surrogate_cells"], "fallback": d_acc["fallback_cells"],
                                "imc": d_acc["imc_cells"]}}
        del g64

    # e2e through the C ABI with host buffers (pinned): every step copies the
    # whole state in and the new state out (mhd_step_host)
    pin_U = torch.empty((8,) + tuple(st.U.shape[1:]), dtype=torch.float64, pin_memory=True).numpy()
    pin_S = torch.empty((8,) + tuple(st.U.shape[1:]), dtype=torch.float64, pin_memory=True).numpy()
    pin_U[...] = st.U
    pin_S[...] = st.species
    out_U = torch.empty(pin_U.shape, dtype=torch.float64, pin_memory=True).numpy()
    out_S = torch.empty(pin_S.shape, dtype=torch.float64, pin_memory=True).numpy()
    g = g32

    def e2e_step():
        # mhd_step_host: the state in from pinned host memory, one step, the
        # new state back (copies of finished arrays overlap the step's tail)
        g.step_host(pin_U, pin_S, out_U, out_S)

    e2e_step()   # untimed: first touch of the pinned buffers
    barrier()
    # each step timed on its own (the call returns with the new state in the
    # host buffers); the host side of this path shows occasional stalls of
    # tens of ms that have nothing to do with the step, so the value is the
    # median step and the mean and every sample are reported beside it
    e2e_ms = []
    for _ in range(12):
        t0 = time.perf_counter()
        e2e_step()
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    barrier()
    e2e_s = float(np.median(e2e_ms)) * 1e-3
    nb = 8 * pin_U.size
    e2e = {"value": world * n3 / e2e_s, "unit": "zone-updates/s", "h2d_bytes_per_step": 2 * nb,
           "d2h_bytes_per_step": 2 * nb, "estimator": "median of 12 steps",
           "ms_per_step_median": e2e_s * 1e3, "ms_per_step_mean": float(np.mean(e2e_ms)),
           "samples_ms": [round(x, 2) for x in e2e_ms]}

    stiff = None if args.no_stiff else stiff_comparison()


    def drift(d0, d1, scale):
        """Mass and momentum change over a run; momentum relative to the sum
        of rho |v| dV of the initial state."""
        return {"mass_rel": (d1["mass"] - d0["mass"]) / d0["mass"],
                "momentum_rel": [(b - a) / scale for a, b in zip(d0["momentum"], d1["momentum"])],
                "divb_max": d1["divb_max"]}

    def rho_absv(state):
        c = (slice(2, -2),) * 3
        dV = float(state.dx[2] * state.dy[2] * state.dz[2])
        return sum(float((state.U[0][c] * np.abs(state.U[q][c])).sum()) for q in (1, 2, 3)) * dV

    # self-gravity (ifgrv = 2): the same chosen-form step with the potential
    # solve and the two half kicks, against the step without them
    grav = None
    if not args.no_gravity:
        sg = st.copy()
        sg.params = st.params.replace(ifgrv=2)
        gg, msg, phg, _, _ = timed_run(native.PREC_FP32, native.COOL_SURROGATE, state=sg, steps=5, warmup=args.warmup)
        grav = {"workload": f"the headline problem with self-gravity, {args.n}^3", "steps": 5,
                "ms_per_step_with_gravity": msg / 5, "ms_per_step_without": ms32 / args.steps,
                "phase_ms": {k: v for k, v in phg.items() if k.startswith("gravity")},
                "potential_solve": "radix-4 FFTs in y (two real z rows per complex transform) and z over the half spectrum, a tridiagonal x solve per mode from tabulated coefficients (FP64)"}
        del gg

    # config 2: 128^3 decaying Mach-5 MHD turbulence, plain FP64, steps 1..100
    # at CFL 0.4 (the timed steps start from the initial state), and the
    # chosen form over the same steps; L1 at the FP64 run's final time
    config2 = None
    if not args.no_config2:
        t2 = problems.turbulence(128)
        n2 = 128 ** 3
        g2, ms2, ph2, _, _ = timed_run(native.PREC_FP64, state=t2, steps=100, warmup=args.warmup, fresh=True)
        gc, msc, phc, _, _ = timed_run(native.PREC_FP32, state=t2, steps=100, warmup=args.warmup, fresh=True)
        sc2 = rho_absv(t2)
        d64, dc = g2.diagnostics(), gc.diagnostics()
        t_end = g2.time
        gc.evolve(20, tsave=t_end)
        Uc, _, bc_ = gc.download()
        U6, _, b6 = g2.download()
        c = (slice(2, -2),) * 3

        def l1r(a, b):
            return float(np.abs(a - b).mean() / np.abs(b).mean())
        config2 = {"workload": "decaying MHD turbulence 128^3, periodic, rms Mach 5, beta 1, k^-4 on |k| = 1..8 "
                               "(ran0 seed 1), CFL 0.4, no cooling, DISSIP off",
                   "steps": 100, "steps_start_from": "t = 0 (a fresh upload after the warm-up)",
                   "plain_fp64": {"value": n2 * 100 / (ms2 * 1e-3), "unit": "zone-updates/s",
                                  "ms_per_step": ms2 / 100, "phase_ms": ph2, "time": t_end,
                                  "conservation": drift(g2.diag0, d64, sc2)},
                   "chosen_form": {"value": n2 * 100 / (msc * 1e-3), "unit": "zone-updates/s",
                                   "ms_per_step": msc / 100, "phase_ms": phc,
                                   "conservation": drift(gc.diag0, dc, sc2),
                                   "l1_vs_fp64_at_same_time": {"rho": l1r(Uc[0][c], U6[0][c]),
                                                               "p": l1r(Uc[4][c], U6[4][c]),
                                                               "B": l1r(bc_[(slice(None),) + c], b6[(slice(None),) + c]),
                                                               "time": gc.time}},
                   "momentum_note": "the reference's MOC limiter reads the energy-based T inside a pencil and "
                                    "the pre-sweep pressure in its ghosts, so at Mach 5 a periodic interface "
                                    "can get two different slopes; the drift is the reference's own (the FP64 "
                                    "path equals the oracle bit for bit)"}
        del g2, gc

    # config 5: the 512^3 colliding flow (10 pc perturbation scale) in the
    # chosen form with the trained surrogate, steps 1..100 with event times
    # per phase, and the plain FP64 path at the same size (3 steps)
    config5 = None
    if not args.no_config5:
        st5 = problems.colliding_flows(512, pert_scale=10.0)
        n5 = 512 ** 3
        g5, ms5, ph5, launches5, clk5 = timed_run(native.PREC_FP32, native.COOL_SURROGATE, state=st5, steps=100,
                                                 warmup=args.warmup, fresh=True)
        d5 = g5.diagnostics()
        divb512 = divb_split(g5, st5)
        d50 = g5.diag0
        del g5
        g5b, ms5b, ph5b, _, _ = timed_run(native.PREC_FP64, state=st5, steps=3, warmup=1)
        del g5b
        config5 = {"workload": "colliding WNM flows with KI cooling, 512^3, 20 pc box, 10 pc perturbation scale, "
                               "free x / periodic y,z",
                   "chosen_form": {"value": n5 * 100 / (ms5 * 1e-3), "unit": "zone-updates/s", "steps": 100,
                                   "ms_per_step": ms5 / 100, "gpu_launches": launches5, "clocks": clk5,
                                   "phases": phase_roofline(ph5, n5, hbm),
                                   "step_frac_of_measured_hbm": B_ALG_STEP * n5 * 100 / (ms5 * 1e-3) / 1e9 / hbm,
                                   "surrogate_cells": d5["surrogate_cells"], "fallback_cells": d5["fallback_cells"],
                                   "imc_cells": d5["imc_cells"], "divb_max": d5["divb_max"],
                                   "divb_max_away_from_free_x_boundaries": divb512[1],
                                   "mass_change_rel": (d5["mass"] - d50["mass"]) / d50["mass"]},
                   "plain_fp64": {"value": n5 * 3 / (ms5b * 1e-3), "unit": "zone-updates/s", "steps": 3,
                                  "ms_per_step": ms5b / 3, "phases": phase_roofline(ph5b, n5, hbm)},
                   "resident_gb": {"fp64_state_and_scratch": 28 * 8 * 516 ** 3 / 1e9,
                                   "fp32_scratch": 15 * 4 * 516 ** 3 / 1e9}}
        config5["speedup_vs_fp64"] = config5["chosen_form"]["value"] / config5["plain_fp64"]["value"]

    if rank != 0:
        return
    sweep_ms = sum(sw32) / len(sw32)
    achieved = B_ALG_SWEEP * n3 / (sweep_ms * 1e-3) / 1e9
    tr = ncu_traffic()
    roof = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
            "traffic": tr * n3 if tr else None, "kernel": "sweep32_kernel (fused RHS+MOC+REMAP, FP32 recon/flux + FP64 accumulation)",
            "peak_source": f"{which} (MEASURED_PEAKS.json hbm_gbs)" if which == "measured" else which,
            "algorithmic_bytes_per_zone": B_ALG_SWEEP}
    if tr:
        # the bytes the kernel really moves (the species too), over the same time
        roof["traffic_gbs"] = tr * n3 / (sweep_ms * 1e-3) / 1e9
        roof["traffic_frac"] = roof["traffic_gbs"] / hbm
    issue = profile_value("sweep_fp32_traffic.txt", "sweep_fp32_issue_active_pct")
    if issue:
        roof["limiter"] = {"issue_active_pct": issue,
                           "fp64_pipe_pct": profile_value("sweep_fp32_traffic.txt", "sweep_fp32_fp64_pipe_pct"),
                           "source": "ncu --set full of the three sweep launches at 128^3 (profiles/)"}
    line = {"metric": "zone-updates/s, 256^3 MHD+KI cool: FP32+surrogate vs plain FP64 at stated L1 err",
            "value": value, "unit": "zone-updates/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms32 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 recon/flux + f64 accumulation",
            "data": "synthetic",
            "config": {"workload": f"colliding WNM flows with KI cooling, {args.n}^3, free x / periodic y,z",
                       "n": args.n, "precision": "fp32 reconstruction+flux, fp64 accumulation",
                       "cooling": "KI surrogate MLP (BF16 tensor cores) + Newton polish, IMC fallback",
                       "l2": "inputs larger than L2 (%.1f GB of FP64 arrays resident, no flush)" % (28 * 8 * (args.n + 4) ** 3 / 1e9),
                       "parallelism": f"replicas x{world}"},
            "plain_fp64": fp64, "l1_error": l1, "stiff_cooling_source": stiff, "speedup_vs_fp64": (value / fp64["value"]) if fp64 else None,
            "fp32_exact_cooling": {"value": n3 * args.steps / (msx * 1e-3), "unit": "zone-updates/s",
                                   "imc_cells": dx_["imc_cells"]},
            "surrogate": {"train_s": sur_train_s, "steps": args.sur_steps, "n_data": args.sur_data,
                          "batch": 65536, "final_mse": float(np.mean(hist[-20:])) if len(hist) else None,
                          "surrogate_cells": d32["surrogate_cells"], "fallback_cells": d32["fallback_cells"],
                          "imc_cells": d32["imc_cells"],
                          "fallback_fraction": (d32["fallback_cells"] / max(1, d32["fallback_cells"] + d32["surrogate_cells"]))},
            "step_zone_updates_roof": hbm * 1e9 / B_ALG_STEP,
            "e2e": e2e, "gpu_launches": launches32, "roofline": roof, "clocks": clocks,
            "phases": phase_roofline(ph32, n3, hbm), "fp64_peak_measured": fp64_peak,
            "diagnostics": {"divb_max": d32["divb_max"], "divb_max_away_from_free_x_boundaries": divb256[1],
                            "mass_change_rel": (d32["mass"] - g32.diag0["mass"]) / g32.diag0["mass"],
                            "note": "x boundaries are open (free): mass changes by the boundary flux, and the "
                                    "reference's face exchange rewrites face n+1, so only the cells next to a free "
                                    "x boundary carry a div B above round-off"},
            "config2": config2, "config5": config5, "self_gravity": grav}
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline()
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
