"""Benchmark: SPH pair-interactions/s of the CheapSynchronousRK2 hydro step.

Workload (default): 3-D Kelvin-Helmholtz in a periodic unit cube, two
lattices of 112 and 142 nodes per unit length (2,134,108 nodes, the nearest
two-lattice set to 128^3 with a 2^(-1/3) spacing ratio), nPerh 1.51, Monaghan-
Gingold Q (Cl = Cq = 1), compatible energy, RigorousSumDensity, CFL 0.5.  One
step = one full CheapSynchronousRK2 step (neighbour build, density sum, dt,
half-step update, mid-point pair loop + smoothing scale, compatible-energy
sweep, full update, boundary enforcement).

value  = unordered neighbour pairs per step x steps / device time of the timed
         steps (state resident in HBM; CUDA events on the library stream).
e2e    = the same metric through the C ABI with host buffers: every step
         uploads the state from pinned host memory (sphgpu_upload_state), runs
         the step, and downloads the new state (sphgpu_download_state).

--impl reference times the CPU implementation of the same step (the oracle's
FP64/OpenMP restatement of the reference loops, all host threads) on a
bounded sample of the workload.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import numpy as np

METRIC = "SPH pair-interactions/sec at stated energy error: mixed vs FP64 GPU vs CPU"
UNIT = "pair-interactions/s"
FLOP_PER_PAIR = 456        # algorithmic FLOPs of the reference pair body per unordered pair
VALUES_PER_NODE = 63       # per-node state read + derivatives written by the pair loop
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per unordered pair
# of one pairKernelFP32 launch, from an ncu --set full capture of
# kelvin_helmholtz(n1=64) (862 MB for 21.76 M pairs); traffic grows in
# proportion to the pairs, so it is scaled by the pairs of the launch.
TRAFFIC_BYTES_PER_PAIR = {"fp32": 39.6}
TRAFFIC_SOURCE = "ncu capture at n1=64 scaled by pairs per launch"


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), "measured", d
    return 6800.0, "fallback", {}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if parts[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["not sampled"], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if ws > 1:
        import torch
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
    return ws, rank, local, dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def make_workload_name(args):
    return None, {"kh": "kelvin_helmholtz_3d", "sweep": "sweep_box", "sod": "sod_planar_3d",
                  "evrard": "evrard_collapse_3d", "asph": "asph_stretched_lattice_3d",
                  "crksph": "kelvin_helmholtz_3d_crksph"}[args.workload]


def asph_box(n1, seed=13):
    """ASPHClassicSmoothingScale workload: the anisotropic jittered lattice
    (spacings 1 : 1.25 : 1.6 across x y z) with rotated tensor H."""
    from spheral_gb300 import problems
    return problems.stretched_box(nx=int(round(1.25 * n1)), ny=n1, nz=int(round(0.8 * n1)), seed=seed)


def crksph_kh(n1):
    """The Kelvin-Helmholtz slab under CRKSPH (LinearOrder, RKSumVolume) as
    the reference's own 3-D test sets it up
    (tests/functional/Hydro/KelvinHelmholtz/KelvinHelmholtz-3d.py with
    CRKSPH=True: MonaghanGingoldViscosity Cl = Cq = 1, no XSPH, interfaces
    smoothed over 0.025, CFL 0.5).  With the CRKSPH() factory's limited Q
    (Cl = 1, Cq = 0.25) and XSPH instead, this slab runs negative specific
    energies after t ~ 0.3-1 in the oracle and on the GPU alike."""
    from spheral_gb300 import problems
    p = problems.kelvin_helmholtz(n1=n1, smooth=0.025)
    p.config.update(hydro="crksph", rk_volume="sum", xsph=False, gradh_correction=False,
                    viscosity="monaghan_gingold", Cl=1.0, Cq=1.0)
    return p


def make_workload(args):
    from spheral_gb300 import problems
    if args.workload == "kh":
        return problems.kelvin_helmholtz(n1=args.n1), "kelvin_helmholtz_3d"
    if args.workload == "sweep":
        return problems.sweep_box(n_side=args.n1, neighbors=args.neighbors), "sweep_box"
    if args.workload == "sod":
        return problems.sod(nx1=args.n1), "sod_planar_3d"
    if args.workload == "evrard":
        return problems.evrard(n=args.n_evrard), "evrard_collapse_3d"
    if args.workload == "asph":
        return asph_box(args.n1), "asph_stretched_lattice_3d"
    if args.workload == "crksph":
        return crksph_kh(args.n1), "kelvin_helmholtz_3d_crksph"
    raise SystemExit("unknown workload")


def cpu_baseline(args, steps=None, warmup=1, n1=None, threads=0):
    """Oracle CheapRK2 steps on a bounded sample of the workload (same
    generator, smaller lattice); returns pairs/s and the sample description.
    threads = 0 uses every host thread, 1 a single core."""
    from oracle import oracle as orc
    from spheral_gb300 import problems
    orc.build()
    n1 = args.cpu_n1 if n1 is None else n1
    orc.set_threads(threads if threads > 0 else (os.cpu_count() or 1))
    if args.workload == "kh":
        p = problems.kelvin_helmholtz(n1=n1)
    elif args.workload == "sweep":
        p = problems.sweep_box(n_side=n1, neighbors=args.neighbors)
    elif args.workload == "evrard":
        p = problems.evrard(n=65536 if threads != 1 else 8192)
    elif args.workload == "asph":
        p = asph_box(n1)
    elif args.workload == "crksph":
        p = crksph_kh(n1)
    else:
        p = problems.sod(nx1=n1)
    o = orc.Oracle(p)
    o.initialize()
    for _ in range(max(1, warmup)):   # the first step allocates
        o.step()
    steps = args.cpu_steps if steps is None else steps
    t0 = time.perf_counter()
    pairs = 0
    for _ in range(steps):
        o.step()
        pairs += o.L.orc_num_pairs(o.h)
    dt = time.perf_counter() - t0
    cores = orc.num_threads()
    orc.set_threads(os.cpu_count() or 1)
    return pairs / dt, dict(n=p.n, n1=n1, steps=steps, seconds=dt, pairs_per_step=pairs / steps,
                            cores=cores, kind="port")


def run_reference(args, ws, rank, dist):
    if rank != 0:
        return
    val, info = cpu_baseline(args, steps=args.steps, warmup=args.warmup)
    sample = (f"{info['steps']} CheapSynchronousRK2 steps of the same generator at n1={args.cpu_n1} "
              f"({info['n']} nodes, {info['pairs_per_step']:.0f} pairs/step), {info['seconds']:.1f} s")
    _, wname = make_workload_name(args)
    line = {
        "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": ws, "steps": info["steps"], "warmup": args.warmup,
        "ms_per_step": 1e3 * info["seconds"] / info["steps"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generator, no external data)",
        "impl": "reference",
        "config": {"workload": wname, "sample_n": info["n"], "sample_n1": args.cpu_n1},
        "cpu_baseline": {"value": val, "unit": UNIT, "cores": info["cores"], "kind": info["kind"], "sample": sample},
        "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def time_steps(eng, steps, prof_names=()):
    eng.profile_reset()
    l0 = eng.launch_count()
    eng.synchronize()
    pairs = 0
    eng.timer_start()
    for _ in range(steps):
        eng.step()
        pairs += eng.neighbor_entries() // 2
    ms = eng.timer_stop()
    launches = eng.launch_count() - l0
    prof = {n: eng.profile_get(n) for n in prof_names}
    return ms, pairs, launches, prof


def kh_mode_amplitude(pos, vel, mass):
    """Amplitude of the vy mode at the seeded wavenumber 4 pi along x at the
    two shear layers y = 0.25 and 0.75 (the growth diagnostic of McNally,
    Lyra and Passy 2012, ApJS 201:18, eqs. 10-13): s, c and d are sums over
    nodes of vy sin(4 pi x) e, vy cos(4 pi x) e and e, with the weight
    e = exp(-4 pi |y - 0.25|) below y = 0.5 and exp(-4 pi |(1 - y) - 0.25|)
    above; the amplitude is 2 sqrt((s/d)^2 + (c/d)^2)."""
    x, y, vy = pos[:, 0], pos[:, 1], vel[:, 1]
    e = np.where(y < 0.5, np.exp(-4.0 * math.pi * np.abs(y - 0.25)), np.exp(-4.0 * math.pi * np.abs(0.75 - y)))
    w = mass * e
    d = np.sum(w)
    s_ = np.sum(w * vy * np.sin(4.0 * math.pi * x)) / d
    c_ = np.sum(w * vy * np.cos(4.0 * math.pi * x)) / d
    return float(2.0 * math.sqrt(s_ * s_ + c_ * c_))


def fp32_vs_fp64(args, local):
    """The mixed mode against an all-FP64 run of the same Kelvin-Helmholtz
    problem at the same physical time.  The FP64 run takes
    args.fp64_compare_steps steps and defines the goal time T; the mixed run
    and a control FP64 run whose initial positions are moved by one ulp are
    advanced to T exactly (the last step is cut at T).  Node-by-node L1 and
    L2 relative differences of rho, eps and v (nodes in the caller's order,
    so the comparison is Lagrangian) and the shear-layer mode amplitude are
    reported for mixed vs FP64 and for the control vs FP64: KH is chaotic, and
    the control measures how far two FP64 runs drift apart from a rounding-
    level change of the initial state."""
    from spheral_gb300.engine import Engine
    prob = crksph_kh(args.compare_n1) if args.workload == "crksph" else None
    if prob is None:
        from spheral_gb300 import problems
        prob = problems.kelvin_helmholtz(n1=args.compare_n1)

    def run(p, precision, goal=None):
        e = Engine.from_problem(p, precision=precision, device=local)
        e.initialize()
        c0 = e.conservation()
        t0 = time.perf_counter()
        steps = 0
        if goal is None:
            e.advance(args.fp64_compare_steps)
            steps = args.fp64_compare_steps
        else:
            while e.time < goal * (1.0 - 1e-15) and steps < 20 * args.fp64_compare_steps:
                e.step(goal)
                steps += 1
        e.synchronize()
        wall = time.perf_counter() - t0
        c1 = e.conservation()
        out = dict(rho=e.field("massDensity"), eps=e.field("specificThermalEnergy"), vel=e.field("velocity"),
                   pos=e.field("position"), t=e.time, steps=steps, wall=wall,
                   err=abs(c1[7] - c0[7]) / abs(c0[7]))
        e.close()
        return out

    ref = run(prob, "fp64")
    goal = ref["t"]
    mixed = run(prob, "fp32", goal)
    import copy
    pert = copy.copy(prob)
    pert.pos = np.ascontiguousarray(np.nextafter(prob.pos, np.inf))
    ctrl = run(pert, "fp64", goal)
    # second control: the FP64 run from initial positions rounded to FP32, a
    # perturbation of the size the mixed mode's FP32 sweeps make at each step
    r32 = copy.copy(prob)
    r32.pos = np.ascontiguousarray(prob.pos.astype(np.float32).astype(np.float64))
    ctrl32 = run(r32, "fp64", goal)

    def diffs(a, b):
        out = {}
        for k in ("rho", "eps", "vel"):
            x, y = a[k].ravel(), b[k].ravel()
            out["L1_" + k] = float(np.sum(np.abs(x - y)) / np.sum(np.abs(y)))
            out["L2_" + k] = float(math.sqrt(np.sum((x - y) ** 2) / np.sum(y * y)))
            out["max_" + k] = float(np.max(np.abs(x - y)) / np.max(np.abs(y)))
        return out

    amp = {name: kh_mode_amplitude(r["pos"], r["vel"], prob.mass) for name, r in
           (("fp64", ref), ("mixed", mixed), ("control", ctrl), ("control_fp32_start", ctrl32))}
    amp0 = kh_mode_amplitude(prob.pos, prob.vel, prob.mass)
    return {"workload": ("kelvin_helmholtz_3d_crksph" if args.workload == "crksph" else "kelvin_helmholtz_3d"),
            "n1": args.compare_n1, "n": prob.n, "goal_time": goal, "steps_fp64": ref["steps"],
            "steps_mixed": mixed["steps"], "steps_control": ctrl["steps"], "steps_control_fp32_start": ctrl32["steps"],
            "time_mixed": mixed["t"], "time_control": ctrl["t"], "time_control_fp32_start": ctrl32["t"],
            "energy_error_fp64": ref["err"], "energy_error_mixed": mixed["err"], "energy_error_control": ctrl["err"],
            "mixed_vs_fp64": diffs(mixed, ref), "control_vs_fp64": diffs(ctrl, ref),
            "control_fp32_start_vs_fp64": diffs(ctrl32, ref),
            "mode_amplitude": dict(amp, initial=amp0),
            "mode_amplitude_rel_diff_mixed": abs(amp["mixed"] - amp["fp64"]) / amp["fp64"],
            "mode_amplitude_rel_diff_control": abs(amp["control"] - amp["fp64"]) / amp["fp64"],
            "mode_amplitude_rel_diff_control_fp32_start":
                abs(amp["control_fp32_start"] - amp["fp64"]) / amp["fp64"],
            "control": "FP64 run with every initial position moved by one ulp (numpy nextafter toward +inf)",
            "control_fp32_start": "FP64 run with the initial positions rounded to FP32",
            "wall_s": {"fp64": ref["wall"], "mixed": mixed["wall"], "control": ctrl["wall"],
                       "control_fp32_start": ctrl32["wall"]}}


def ensemble_record(args, local, nboxes, steps, warmup=2):
    """Batched-ensemble throughput against one large box of about the same
    total size: nboxes turbulent boxes (counts log-uniform 4,096..262,144,
    seeded) advanced together by sphgpu_ensemble_advance, then one box alone."""
    from spheral_gb300.engine import Engine
    from spheral_gb300 import problems
    import torch
    probs = problems.ensemble(nboxes)
    engines = [Engine.from_problem(p, precision=args.precision, device=local) for p in probs]
    for e in engines:
        e.initialize()
    Engine.ensemble_advance(engines, warmup, nthreads=args.threads)
    e0 = [e.conservation()[7] for e in engines]
    before = sum(e.neighbor_entries() // 2 for e in engines)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    Engine.ensemble_advance(engines, steps, nthreads=args.threads)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    after = sum(e.neighbor_entries() // 2 for e in engines)
    pairs = 0.5 * (before + after) * steps
    value = pairs / wall
    errs = [abs(e.conservation()[7] - a) / abs(a) for e, a in zip(engines, e0)]
    ntot = sum(p.n for p in probs)
    nmin, nmax = min(p.n for p in probs), max(p.n for p in probs)
    for e in engines:
        e.close()
    side = int(round(ntot ** (1.0 / 3.0)))
    big = Engine.from_problem(problems.turbulent_box(side, 1), precision=args.precision, device=local)
    big.initialize()
    big.advance(warmup)
    torch.cuda.synchronize()
    bsteps = max(3, min(steps, 30))
    b_before = big.neighbor_entries() // 2
    t0 = time.perf_counter()
    big.advance(bsteps)
    torch.cuda.synchronize()
    bwall = time.perf_counter() - t0
    b_pairs = 0.5 * (b_before + big.neighbor_entries() // 2) * bsteps
    single = b_pairs / bwall
    big.close()
    return {"boxes": nboxes, "n_total": ntot, "n_min": nmin, "n_max": nmax, "steps": steps, "value": value,
            "unit": UNIT, "wall_s": wall, "energy_error_max_over_boxes": max(errs),
            "single_large_run": {"n": side ** 3, "value": single, "unit": UNIT, "steps": bsteps},
            "ensemble_over_single": value / single,
            "timer": "host wall clock, device synchronised on both sides"}


def pipe_peak_tflops(precision, sm_count, sm_mhz):
    """Nominal non-tensor FMA peak: FP32 128 lanes per SM, FP64 at GB300's
    nominal 1.25 TFLOP/s for 152 SMs at 2,070 MHz (about 2 FP64 lanes per SM),
    each lane 2 FLOP per clock, scaled by the device's SM count and max clock."""
    lanes = 128.0 if precision == "fp32" else 1.25e12 / (152 * 2 * 2070e6)
    return sm_count * lanes * 2.0 * sm_mhz * 1e6 / 1e12


def run_ours(args, ws, rank, local, dist):
    from spheral_gb300.engine import Engine
    prob, wname = make_workload(args)
    n = prob.n
    eng = Engine.from_problem(prob, precision=args.precision, device=local)
    if args.search_width:
        eng.set_neighbor_width(args.search_width)
    if args.pair_variant >= 0:
        eng.set_pair_variant(args.pair_variant)
    eng.initialize()
    for _ in range(args.warmup):
        eng.step()
    e0 = eng.conservation()
    f32 = args.precision in ("fp32", "fp32_plain")
    pair_kernel = "pair_crk" if args.workload == "crksph" else ("pair_fp32" if f32 else "pair_fp64")
    names = [pair_kernel, "rk_corrections", "rk_volume", "gravity", "neighbor_count", "neighbors", "neighbor_items", "sum_density", "density_dt", "dt",
             "energy",
             "gradh", "radix_sort",
             "permute", "update", "prepare_fp32", "enforce", "cell_keys", "bounds", "cell_ranges"]
    eng.profile(True)
    barrier(dist)
    with ClockSampler(local) as clk:
        ms, pairs, launches, prof = time_steps(eng, args.steps, names)
    eng.profile(False)
    ms = max_over_ranks(dist, ms)
    pair_variant = eng.pair_variant()[0] if f32 else None
    nb_width = eng.neighbor_width()   # lanes per group of the neighbour search (autotuned)
    e1 = eng.conservation()
    energy_err = abs(e1[7] - e0[7]) / abs(e0[7])
    p_scale = float(np.sum(prob.mass * np.linalg.norm(prob.vel, axis=1)))   # sum m |v| of the initial state
    mom_err = float(np.linalg.norm(e1[1:4] - e0[1:4]) / p_scale) if p_scale > 0 else None
    value = ws * pairs / (ms / 1e3)
    k_mean = 2.0 * pairs / args.steps / n

    # e2e through the C ABI with host buffers
    import torch
    pin = lambda shape: torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()
    hp, hv, hr, he, hH = pin((n, 3)), pin((n, 3)), pin(n), pin(n), pin((n, 6))
    hm = pin(n)
    hm[:] = prob.mass
    eng.download_state(hp, hv, hr, he, hH)
    barrier(dist)
    eng.synchronize()
    e2e_pairs = 0
    eng.timer_start()
    for _ in range(args.e2e_steps):
        eng.upload_state(hp, hv, hm, hr, he, hH)
        eng.step()
        e2e_pairs += eng.neighbor_entries() // 2
        eng.download_state(hp, hv, hr, he, hH)
    e2e_ms = max_over_ranks(dist, eng.timer_stop())
    e2e_value = ws * e2e_pairs / (e2e_ms / 1e3)
    h2d = n * (3 + 3 + 1 + 1 + 1 + 6) * 8
    d2h = n * (3 + 3 + 1 + 1 + 6) * 8

    # FP64 GPU comparison (same workload, same step) for the mixed-vs-FP64 ratio
    fp64 = None
    if args.precision == "fp32" and args.fp64_steps > 0:
        e64 = Engine.from_problem(prob, precision="fp64", device=local)
        e64.initialize()
        for _ in range(args.warmup):
            e64.step()
        names64 = ["pair_crk" if args.workload == "crksph" else "pair_fp64"]
        e64.profile(True)
        ms64, pairs64, _, prof64 = time_steps(e64, args.fp64_steps, names64)
        e64.profile(False)
        n64, t64 = prof64[names64[0]]
        fp64 = {"value": pairs64 / (ms64 / 1e3), "unit": UNIT, "steps": args.fp64_steps,
                "ms_per_step": ms64 / args.fp64_steps, "pair_kernel_ms": t64 / max(1, n64),
                "pairs_per_launch": pairs64 / args.fp64_steps}
        e64.close()

    # Energy-conservation error of the mixed-precision run over a long run:
    # keep stepping the same engine to energy_steps steps after warm-up.
    done = args.steps + args.e2e_steps
    for _ in range(max(0, args.energy_steps - done)):
        eng.step()
    e_end = eng.conservation()
    long_steps = max(done, args.energy_steps)
    long_err = abs(e_end[7] - e0[7]) / abs(e0[7])
    long_mom = float(np.linalg.norm(e_end[1:4] - e0[1:4]) / p_scale) if p_scale > 0 else None

    # Accuracy of the mixed mode against an all-FP64 run of the same problem
    # at the same physical time, with an FP64 chaos control.
    compare = None
    if args.fp64_compare_steps > 0 and args.precision == "fp32" and args.workload in ("kh", "crksph"):
        compare = fp32_vs_fp64(args, local)

    ens = None
    if args.ens_boxes > 0 and args.workload == "kh":
        ens = ensemble_record(args, local, args.ens_boxes, args.ens_steps)

    if rank != 0:
        return
    hbm, peak_kind, pk = peaks()
    nl, tl = prof.get(pair_kernel, (0, 0.0))
    avg_ms = tl / max(1, nl)
    pairs_per_launch = pairs / max(1, args.steps)
    elem = 4 if f32 else 8
    b_pair = elem * VALUES_PER_NODE / (k_mean / 2.0) + 6 * elem
    achieved_gbs = b_pair * pairs_per_launch / (avg_ms / 1e3) / 1e9 if avg_ms > 0 else None
    tflops = FLOP_PER_PAIR * pairs_per_launch / (avg_ms / 1e3) / 1e12 if avg_ms > 0 else None
    clocks = clk.summary()
    sm_count = torch.cuda.get_device_properties(local).multi_processor_count
    pipe = "fp32" if f32 else "fp64"
    pipe_peak = pipe_peak_tflops(pipe, sm_count, clocks["sm_max_mhz"] or 2070.0)
    if fp64 is not None and fp64["pair_kernel_ms"] > 0:
        fp64["pair_kernel_tflops"] = FLOP_PER_PAIR * fp64["pairs_per_launch"] / (fp64["pair_kernel_ms"] / 1e3) / 1e12
        fp64["fp64_pipe_peak_tflops"] = pipe_peak_tflops("fp64", sm_count, clocks["sm_max_mhz"] or 2070.0)
        fp64["fp64_pipe_frac"] = fp64["pair_kernel_tflops"] / fp64["fp64_pipe_peak_tflops"]
    cpu = None
    if args.cpu_steps > 0:
        cval, cinfo = cpu_baseline(args)
        cpu = {"value": cval, "unit": UNIT, "cores": cinfo["cores"], "kind": "port",
               "sample": (f"{cinfo['steps']} steps of the same generator at n1={cinfo['n1']} ({cinfo['n']} nodes), "
                          f"{cinfo['seconds']:.1f} s, FP64 oracle, OpenMP on every host thread"),
               "build": "g++ -O3 -fopenmp -ffp-contract=off (no -march=native: the oracle must give the same "
                        "results on the x86-64 and aarch64 hosts)"}
        if args.cpu1_steps > 0:
            v1, i1 = cpu_baseline(args, steps=args.cpu1_steps, n1=args.cpu1_n1, threads=1)
            cpu["one_core"] = {"value": v1, "unit": UNIT, "cores": i1["cores"],
                               "sample": (f"{i1['steps']} steps at n1={i1['n1']} ({i1['n']} nodes), "
                                          f"{i1['seconds']:.1f} s, one thread")}
    line = {
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "fp32" if f32 else "f64",
        "precision": {"fp32": ("FP32 pair sweeps on cell-relative positions with compensated sums; FP64 neighbour "
                               "criterion, integration, compatible energy and tallies"),
                      "fp32_plain": ("FP32-relative: FP32 pair sweeps on cell-relative positions with plain "
                                     "(uncompensated) sums; FP64 neighbour criterion, integration and tallies"),
                      "fp64": "FP64 throughout"}[args.precision],
        "data": "synthetic (seeded generator, no external data)",
        "energy_error": long_err,
        "energy_error_steps": long_steps,
        "energy_error_timed_steps": energy_err,
        "momentum_error": long_mom,
        "momentum_error_timed_steps": mom_err,
        "momentum_error_definition": "|P(t) - P(0)| / sum m |v(0)|",
        "fp32_vs_fp64": compare,
        "config": {"workload": wname, "n": n, "n1": prob.meta.get("n1"), "n2": prob.meta.get("n2"),
                   "mean_neighbors": k_mean, "pairs_per_step": pairs / args.steps,
                   "cache": "inputs larger than L2 (state + neighbour lists > 1 GB)",
                   "parallelism": f"replicas x{ws}"},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "steps": args.e2e_steps},
        "gpu_launches": launches,
        "pair_variant": pair_variant,
        "neighbor_width": nb_width,
        "roofline": {"bound": f"{pipe}_pipe", "achieved": tflops, "peak": pipe_peak, "unit": "TFLOP/s",
                     "frac": (tflops / pipe_peak) if tflops else None,
                     "traffic": (TRAFFIC_BYTES_PER_PAIR[pipe] * pairs_per_launch
                                 if pipe in TRAFFIC_BYTES_PER_PAIR else None),
                     "traffic_source": TRAFFIC_SOURCE,
                     "peak_kind": (f"nominal non-tensor {pipe.upper()} FMA rate: {sm_count} SMs (queried) x "
                                   f"{'128' if f32 else '~2'} lanes x 2 FLOP x max SM clock; no "
                                   "FP32/FP64 pipe figure is in the measured peaks"),
                     "kernel": pair_kernel, "flop_per_pair": FLOP_PER_PAIR, "pairs_per_launch": pairs_per_launch,
                     "avg_launch_ms": avg_ms, "sm_count": sm_count,
                     "why": ("pairs/s roof = min(pipe / 456 FLOP, HBM / B_pair); the pipe roof is the lower one for "
                             "this mode, so it binds"),
                     "hbm": {"achieved": achieved_gbs, "peak": hbm, "unit": "GB/s", "peak_kind": peak_kind,
                             "frac": (achieved_gbs / hbm) if achieved_gbs else None,
                             "algorithmic_bytes_per_pair": b_pair}},
        "kernel_ms_per_step": {k: v[1] / args.steps for k, v in prof.items() if v[0] > 0},
        "fp64_gpu": fp64,
        "ensemble": ens,
        "cpu_baseline": cpu,
        "clocks": clocks,
    }
    print(json.dumps(line), flush=True)


def run_ensemble(args, ws, rank, local, dist):
    """Batched ensemble: args.boxes turbulent boxes with log-uniform particle
    counts (4,096 to 262,144, seeded), all advanced by sphgpu_ensemble_advance
    (one stream per box, host threads feeding them), against one large box
    of about the same total size advanced alone."""
    from spheral_gb300.engine import Engine
    import torch
    probs = problems_ensemble(args.boxes)
    engines = [Engine.from_problem(p, precision=args.precision, device=local) for p in probs]
    for e in engines:
        e.initialize()
    Engine.ensemble_advance(engines, args.warmup, nthreads=args.threads)
    e0 = [e.conservation()[7] for e in engines]
    before = sum(e.neighbor_entries() // 2 for e in engines)
    barrier(dist)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        Engine.ensemble_advance(engines, args.steps, nthreads=args.threads)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    wall = max_over_ranks(dist, wall)
    after = sum(e.neighbor_entries() // 2 for e in engines)
    pairs = 0.5 * (before + after) * args.steps
    value = ws * pairs / wall
    errs = [abs(e.conservation()[7] - a) / abs(a) for e, a in zip(engines, e0)]
    ntot = sum(p.n for p in probs)
    for e in engines:
        e.close()
    # single large box of about the same total size, advanced alone
    from spheral_gb300 import problems
    side = int(round(ntot ** (1.0 / 3.0)))
    big = Engine.from_problem(problems.turbulent_box(side, 1), precision=args.precision, device=local)
    big.initialize()
    big.advance(args.warmup)
    torch.cuda.synchronize()
    bsteps = max(3, min(args.steps, 30))
    b_before = big.neighbor_entries() // 2
    t0 = time.perf_counter()
    big.advance(bsteps)
    torch.cuda.synchronize()
    bwall = time.perf_counter() - t0
    b_pairs = 0.5 * (b_before + big.neighbor_entries() // 2) * bsteps
    single = b_pairs / bwall
    big.close()
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * wall / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "fp32" if args.precision == "fp32" else "f64", "data": "synthetic (seeded generator, no external data)",
        "config": {"workload": f"ensemble_{args.boxes}_turbulent_boxes", "boxes": args.boxes, "n_total": ntot,
                   "n_min": min(p.n for p in probs), "n_max": max(p.n for p in probs),
                   "host_threads": args.threads or os.cpu_count(), "timer": "host wall clock, device synchronised",
                   "parallelism": f"replicas x{ws}"},
        "energy_error_max_over_boxes": max(errs),
        "single_large_run": {"n": side ** 3, "value": single, "unit": UNIT, "steps": bsteps},
        "ensemble_over_single": value / single,
        "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)


def run_evrard_validation(args, ws, rank, local, dist):
    """The Evrard collapse (1,048,576 nodes, mixed mode) integrated to
    t = 0.8 and its radial profiles against the comparison profiles the
    reference ships with its functional test
    (tests/functional/EvrardSphericalCollapse/{rho,vel,entropy}.dat, kept as
    tests/golden/evrard_profiles.npz)."""
    from spheral_gb300 import problems
    from spheral_gb300.engine import Engine
    import torch
    ref = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "tests", "golden", "evrard_profiles.npz"))
    p = problems.evrard(n=args.n_evrard)
    eng = Engine.from_problem(p, precision=args.precision, device=local)
    eng.initialize()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    steps = 0
    while eng.time < args.goal_time * (1.0 - 1e-12) and steps < args.max_steps:
        eng.step(args.goal_time)
        steps += 1
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    t_end = eng.time
    x = eng.field("position")
    v = eng.field("velocity")
    rho = eng.field("massDensity")
    P = eng.field("pressure")
    r = np.linalg.norm(x, axis=1)
    vr = np.sum(v * x, axis=1) / np.maximum(r, 1e-30)
    A = P / rho ** (5.0 / 3.0)
    edges = np.logspace(np.log10(0.01), 0.0, 41)
    mid = np.sqrt(edges[1:] * edges[:-1])
    idx = np.digitize(r, edges) - 1
    prof = {k: np.array([np.median(a[idx == b]) if np.any(idx == b) else np.nan for b in range(len(mid))])
            for k, a in (("rho", rho), ("vel", vr), ("entropy", A))}
    sel = (mid > 0.05) & (mid < 0.7)
    out = {}
    for k in ("rho", "vel", "entropy"):
        rr, vv = ref[k + "_r"], ref[k]
        want = np.interp(np.log(mid[sel]), np.log(rr), vv)
        got = prof[k][sel]
        ok = np.isfinite(got)
        if k == "vel":
            out["L1_vr_over_max"] = float(np.mean(np.abs(got[ok] - want[ok])) / np.max(np.abs(vv)))
        else:
            out["mean_abs_log10_" + k] = float(np.mean(np.abs(np.log10(got[ok] / want[ok]))))
    # kernel split of five more steps past the goal time (profiles above are taken at it)
    names = ["pair_fp32", "pair_fp64", "gravity", "neighbors", "neighbor_items", "density_dt", "gradh", "energy",
             "update", "permute", "radix_sort", "prepare_fp32", "enforce", "cell_keys", "bounds", "cell_ranges", "dt"]
    eng.profile_reset()
    eng.profile(True)
    for _ in range(5):
        eng.step()
    eng.profile(False)
    late = {k: eng.profile_get(k)[1] / 5 for k in names if eng.profile_get(k)[0] > 0}
    if rank != 0:
        return
    line = {"workload": "evrard_collapse_3d", "n": p.n, "goal_time": args.goal_time, "time": t_end, "steps": steps,
            "wall_s": wall, "precision": args.precision, "validation": out, "late_kernel_ms_per_step": late,
            "profile_r": [float(a) for a in mid], "profile_rho": [float(a) for a in prof["rho"]],
            "profile_vr": [float(a) for a in prof["vel"]], "profile_entropy": [float(a) for a in prof["entropy"]]}
    print(json.dumps(line), flush=True)


def problems_ensemble(nboxes):
    from spheral_gb300 import problems
    return problems.ensemble(nboxes)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="kh", choices=["kh", "sweep", "sod", "ensemble", "evrard", "asph", "crksph"])
    ap.add_argument("--n-evrard", type=int, default=1048576)
    ap.add_argument("--validate", action="store_true", help="evrard: integrate to --goal-time and compare profiles")
    ap.add_argument("--goal-time", type=float, default=0.8)
    ap.add_argument("--max-steps", type=int, default=100000)
    ap.add_argument("--boxes", type=int, default=256)
    ap.add_argument("--threads", type=int, default=0)
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp32_plain", "fp64"])
    ap.add_argument("--n1", type=int, default=112)
    ap.add_argument("--neighbors", type=int, default=64)
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--fp64-steps", type=int, default=10)
    ap.add_argument("--energy-steps", type=int, default=1000)
    ap.add_argument("--fp64-compare-steps", type=int, default=1000,
                    help="steps of the FP64 run that sets the goal time of the mixed-vs-FP64 comparison (0: skip)")
    ap.add_argument("--compare-n1", type=int, default=56, help="lattice of the mixed-vs-FP64 comparison")
    ap.add_argument("--ens-boxes", type=int, default=64, help="boxes of the ensemble sub-record (0: skip)")
    ap.add_argument("--ens-steps", type=int, default=20)
    ap.add_argument("--cpu-n1", type=int, default=56)
    ap.add_argument("--cpu-steps", type=int, default=6)
    ap.add_argument("--cpu1-n1", type=int, default=28, help="lattice of the one-core CPU sample")
    ap.add_argument("--cpu1-steps", type=int, default=2)
    ap.add_argument("--search-width", type=int, default=0, choices=[0, 8, 16, 32],
                    help="pin the neighbour-search group width (0: autotuned)")
    ap.add_argument("--pair-variant", type=int, default=-1,
                    help="pin the mixed pair kernel's variant (-1: autotuned)")
    args = ap.parse_args()
    ws, rank, local, dist = dist_setup()
    if args.impl == "reference":
        run_reference(args, ws, rank, dist)
    else:
        from spheral_gb300 import build
        build.build()
        if args.workload == "ensemble":
            run_ensemble(args, ws, rank, local, dist)
        elif args.workload == "evrard" and args.validate:
            run_evrard_validation(args, ws, rank, local, dist)
        else:
            run_ours(args, ws, rank, local, dist)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
