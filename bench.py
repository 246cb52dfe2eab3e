#!/usr/bin/env python3
"""Benchmark of the GB300 Mercurius integrator.

Metric: FP64 body-steps/s (bodies excluding the Sun x steps / second) of the
planetary-embryo disk (Sun + Jupiter/Saturn analogues + 2000 embryos, all
massive, dt 0.01 yr, changeover 3 Hill radii) integrated with the
universal-variable drift.  Synthetic, seeded initial conditions.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

ours:       K timed steps on the GPU through libmerc.so.  One bench step is one
            merc_step call that advances the system by --batch integrator steps
            (default 64: eight replays of the 8-step graph, the kicks at the
            graph boundaries merged; the reference likewise advances
            BATCH_SIZE steps per kernel launch), with the L2 flushed
            (512 MB write) between calls; `value` counts integrator body-steps
            over device time (CUDA events), `e2e` is host wall time of the
            public C-ABI call sequence set_state (H2D, pinned) -> step -> get_state
            (D2H, pinned) per bench step, replaying the timed calls from the
            same start state with the same flush.  Also reported: kick-kernel
            roofline against the measured FP64 FMA peak, the same for the
            encounter sub-step kernel (timed in three more calls), the CPU
            oracle on the host cores (the reference's element step as
            cpu_baseline, the universal drift beside it; for the sweep and the
            Planet Nine workload OpenMP over systems), and the element-drift
            (reference-algorithm) path on the GPU.
reference:  the CPU restatement of the reference's step (element drift,
            oracle/, OpenMP over all host cores), same workload and metric; the
            reference itself is CUDA only and ships no CPU path.
N > 1 runs N independent replicas (one per GPU, no collective; weak scaling).
"""
from __future__ import annotations

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
sys.path.insert(0, os.path.join(ROOT, "p9-integrator_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import systems  # noqa: E402

METRIC = "FP64 body-steps/s (N=2000 embryo disk)"
UNIT = "body-steps/s"
FLOPS_PER_PAIR = 27  # kick work per pair: FMA = 2, sqrt and divide = 1 each


def workload():
    return systems.embryo_disk()


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
        return world, rank, local, dist
    return 1, 0, 0, None


def max_over_ranks(dist, x):
    if dist is None:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(dist, x):
    if dist is None:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                smax = float(f[1])
            except ValueError:
                continue
            for name, val in zip(names, f[4:8]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "samples": len(sm),
                "reasons": sorted(reasons)}


def cpu_rate(sysm, params_kw, sample_s=12.0, warm_steps=0, label=None):
    """The oracle (OpenMP over bodies for one system, over systems for a
    batch) on this host's cores: body-steps/s over a bounded number of steps
    of the full workload, after `warm_steps` untimed steps."""
    from oracle import Oracle
    from oracle import default_params as oparams

    O = Oracle()
    p = oparams(**params_kw)
    pos, vel, alag = O.load_elements(p, sysm.body_offset, sysm.n_massive, sysm.mass, sysm.elements)
    fl = None
    if warm_steps:
        pos, vel, alag, fl, _ = O.run(p, sysm.body_offset, sysm.n_massive, sysm.mass, pos, vel, alag,
                                      steps=warm_steps)
    t0 = time.perf_counter()
    pos, vel, alag, fl, _ = O.run(p, sysm.body_offset, sysm.n_massive, sysm.mass, pos, vel, alag, flags=fl, steps=1)
    one = time.perf_counter() - t0
    steps = int(max(1, min(5000, sample_s / max(one, 1e-6))))
    t0 = time.perf_counter()
    O.run(p, sysm.body_offset, sysm.n_massive, sysm.mass, pos, vel, alag, flags=fl, steps=steps)
    dt = time.perf_counter() - t0
    drift = "element drift (the reference's step)" if params_kw.get("drift", 0) == 0 else "universal drift"
    return {"value": sysm.n_total * steps / dt, "unit": UNIT, "cores": O.threads(), "kind": "port",
            "sample": f"{steps} steps of the full {sysm.n_total}-body workload{label or ''}, {drift} ({dt:.1f} s)"}


def cpu_baseline(sysm, params_kw, sample_s=12.0):
    return cpu_rate(sysm, params_kw, sample_s)


def run_reference(args, world, rank, dist):
    """The reference's algorithm on the host cores: the oracle's restatement
    of the reference step (element drift: elements round trip and 8 fixed
    Danby iterations, src/sim.cuh:692-713), binary64 with the host's C
    library, OpenMP over the bodies; the universal-drift figure beside it."""
    if rank != 0:
        return
    from oracle import Oracle
    from oracle import default_params as oparams

    sysm = workload()
    kw = dict(dt=sysm.dt, hill_factor=sysm.hill_factor, drift=0)
    O = Oracle()
    p = oparams(**kw)
    pos, vel, alag = O.load_elements(p, sysm.body_offset, sysm.n_massive, sysm.mass, sysm.elements)
    S = args.batch
    pos, vel, alag, fl, _ = O.run(p, sysm.body_offset, sysm.n_massive, sysm.mass, pos, vel, alag,
                                  steps=args.warmup * S)
    t0 = time.perf_counter()
    O.run(p, sysm.body_offset, sysm.n_massive, sysm.mass, pos, vel, alag, flags=fl, steps=args.steps * S)
    dt = time.perf_counter() - t0
    value = sysm.n_total * S * args.steps / dt
    universal = cpu_rate(sysm, dict(kw, drift=1), sample_s=8.0, warm_steps=args.warmup * S)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": sysm.label, "bodies": sysm.n_total, "n_massive": int(sysm.n_massive[0]),
                       "dt": sysm.dt, "drift": "elements (the reference's step)", "hill_factor": sysm.hill_factor,
                       "batch": S, "step": f"{S} integrator steps"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": O.threads(), "kind": "port",
                             "sample": f"{args.steps * S} full integrator steps after {args.warmup * S} warm-up "
                                       f"steps, element drift (the reference's step)"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "cpu_universal_drift": universal,
            "note": "CPU restatement of the reference step (src/sim.cuh:679-742, element drift) on all host "
                    "cores; the reference ships CUDA only"}
    print(json.dumps(line), flush=True)


def load_traffic():
    path = os.path.join(ROOT, "profiles", "roofline_traffic.json")
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def sweep_section(merc, args, local, dist, world, rank):
    """Batched sweep (workload 2: 4096 uneven systems in one context, every
    phase one launch over all systems) against the same systems launched one
    by one (one context, load + steps per system, a timed sample of systems).
    Replicas: each rank takes a contiguous share of the systems."""
    full = systems.sweep()
    sysm = systems.shard(full, rank, world)
    kw = dict(dt=sysm.dt, hill_factor=sysm.hill_factor, drift=merc.DRIFT_UNIVERSAL)
    g = merc.Integrator(merc.default_params(**kw), device=local)
    g.load_systems(sysm)
    g.step(args.warmup)
    steps = max(3, min(args.steps, 20))
    # one call of `steps` steps, as a user integrates a sweep; the state
    # (>100 MB of SoA arrays) is larger than L2
    g.step(steps)
    ms = max_over_ranks(dist, g.stats().last_step_ms)
    batched = sum_over_ranks(dist, float(sysm.n_total * steps)) / (ms / 1e3)
    pairs = sysm.pairs_per_step()
    g.close()
    # one by one: a sample of the systems, each loaded and stepped alone,
    # with the plain guess dt / r0
    sample = sysm.subset(np.linspace(0, sysm.n_systems - 1, 48).astype(int))
    g1 = merc.Integrator(merc.default_params(warm_start=merc.WARM_PLAIN, **kw), device=local)
    t_ms, bodies = 0.0, 0
    for s in range(sample.n_systems):
        one = sample.subset([s])
        g1.load_systems(one)
        g1.step(2)
        g1.step(steps)
        t_ms += g1.stats().last_step_ms
        bodies += one.n_total * steps
    g1.close()
    one_by_one = bodies / (t_ms / 1e3)
    return {"workload": full.label, "systems": int(full.n_systems), "bodies": int(full.n_total),
            "steps": steps, "batched_body_steps_per_s": batched, "batched_ms_per_step": ms / steps,
            "batched_pairs_per_s": sum_over_ranks(dist, float(pairs)) * steps / (ms / 1e3),
            "one_by_one_body_steps_per_s": one_by_one, "one_by_one_sample_systems": int(sample.n_systems),
            "one_by_one_guess": "plain dt/r0",
            "speedup_vs_one_by_one": batched / one_by_one}


def sweep_cpu(gpu):
    """The 4096-system sweep on the host cores (OpenMP over systems, the
    reference's ensemble split src/simutils.cuh:288-290 done by threads):
    the universal drift the GPU runs and the reference's element step."""
    sysm = systems.sweep()
    kw = dict(dt=sysm.dt, hill_factor=sysm.hill_factor)
    uni = cpu_rate(sysm, dict(kw, drift=1), sample_s=6.0)
    ele = cpu_rate(sysm, dict(kw, drift=0), sample_s=6.0)
    return {"cpu_universal": uni, "cpu_elements": ele,
            "gpu_over_cpu_universal": gpu["batched_body_steps_per_s"] / uni["value"]}


def p9_cpu():
    """The Planet Nine sweep on the host cores, both drifts (OpenMP over systems)."""
    sysm = systems.p9_sweep()
    kw = dict(dt=sysm.dt, hill_factor=sysm.hill_factor)
    return {"cpu_universal": cpu_rate(sysm, dict(kw, drift=1), sample_s=4.0),
            "cpu_elements": cpu_rate(sysm, dict(kw, drift=0), sample_s=4.0)}


def p9_section(merc, args, local, dist, world, rank):
    """The reference's own workload: the Planet Nine configuration (Planet
    Nine + 4 giants + 10235 TNOs, p9_config.py) as 32 sweep systems in one
    context (the reference runs 4 per device), dt 0.8219, changeover at 1 Hill
    radius; universal drift (persistent kernel) and the reference's element
    drift.  Replicas: each rank takes a share of the systems."""
    full = systems.p9_sweep()
    sysm = systems.shard(full, rank, world)
    out = {"workload": full.label, "systems": int(full.n_systems), "bodies": int(full.n_total)}
    steps = max(3, min(args.steps, 20))
    for name, drift in (("universal", merc.DRIFT_UNIVERSAL), ("elements", merc.DRIFT_ELEMENTS)):
        g = merc.Integrator(merc.default_params(dt=sysm.dt, hill_factor=sysm.hill_factor, drift=drift), device=local)
        g.load_systems(sysm)
        g.step(2)
        g.step(steps)
        ms = max_over_ranks(dist, g.stats().last_step_ms)
        g.close()
        out[name] = {"body_steps_per_s": sum_over_ranks(dist, float(sysm.n_total * steps)) / (ms / 1e3),
                     "ms_per_step": ms / steps, "steps": steps}
    return out


def planetesimal_section(merc, args, local, dist, world, rank, peak):
    """Workload 4: Sun + 4 giants + 8192 planetesimals + 131072 test particles,
    dt 0.25, one 8-step graph (test-particle half kicks merged across step
    boundaries).  Reports body-steps/s, pair interactions/s and the HBM rate of
    the test-particle state stream (96 B per body-step: read and write x, v)."""
    sysm = systems.planetesimal_disk()
    g = merc.Integrator(merc.default_params(dt=sysm.dt, hill_factor=sysm.hill_factor, drift=merc.DRIFT_UNIVERSAL),
                        device=local)
    g.load_systems(sysm)
    g.step(1)
    steps = 8
    g.step(steps)
    ms = max_over_ranks(dist, g.stats().last_step_ms)
    g.close()
    nm = int(sysm.n_massive[0])
    nt = sysm.n_total - nm
    t = ms / 1e3
    return {"workload": sysm.label, "bodies": int(sysm.n_total), "n_massive": nm, "steps": steps,
            "body_steps_per_s": sum_over_ranks(dist, float(sysm.n_total * steps)) / t, "ms_per_step": ms / steps,
            "pairs_per_s": sum_over_ranks(dist, float(2 * (nm * (nm - 1) + nt * nm) * steps)) / t,
            "test_particle_stream_gbs": sum_over_ranks(dist, 96.0 * nt * steps) / t / 1e9,
            "fp64_frac_algorithmic": FLOPS_PER_PAIR * 2 * (nm * (nm - 1) + nt * nm) * steps / t / 1e12 / peak,
            "fp64_frac_note": "27 algorithmic flops per ordered pair and half kick over the measured FP64 FMA "
                              "peak, whole step; above 1 because the two half kicks around a step boundary are "
                              "merged into one pass (18 FP64 instructions per test-particle pair serve 54 "
                              "algorithmic flops) and the symmetric massive pass evaluates each unordered pair "
                              "once"}


def warm_start_section(merc, args, local):
    """Learned warm start of the universal drift: log ~1e7 (drift input ->
    converged anomaly) pairs from the embryo disk, the sweep and a set of hard
    drifts (e up to 0.99 near perihelion, hyperbolic flybys), train the FP32
    MLP on the GPU, then integrate each workload (the planetesimal disk, and a
    hard-drift set drawn with another seed) from the same initial state with
    the plain guess dt/r0, the learned guess and the third-order series guess
    (the default).  Reported per guess: Newton iterations per solve, the
    iterations the warps executed per solve (a warp runs as many iterations as
    its slowest lane), ms per step."""
    c1, c2 = systems.embryo_disk(), systems.sweep()
    hard = systems.hard_drifts(seed=20261212)
    kw = dict(hill_factor=3.0, drift=merc.DRIFT_UNIVERSAL)
    g1 = merc.Integrator(merc.default_params(dt=c1.dt, **kw), device=local)
    g1.load_systems(c1)
    g1.mlp_log(1_000_000)
    g1.step(400)
    log1 = g1.mlp_get_log()
    g1.close()
    g = merc.Integrator(merc.default_params(dt=c2.dt, **kw), device=local)
    g.load_systems(c2)
    g.mlp_log(12_000_000)
    g.step(4)
    g.mlp_append_log(log1)
    gh = merc.Integrator(merc.default_params(dt=hard.dt, **kw), device=local)
    gh.load_systems(hard)
    gh.mlp_log(2_000_000)
    gh.step(4)
    g.mlp_append_log(gh.mlp_get_log())
    gh.close()
    n_log = g.mlp_log_count()
    t0 = time.perf_counter()
    loss = g.mlp_train(epochs=12, batch=16384, lr=3e-3, seed=7)
    train_s = time.perf_counter() - t0
    w = g.mlp_weights()
    g.close()
    out = {"logged_pairs": int(n_log), "train_seconds": train_s, "epochs": 12,
           "loss_first_last": [float(loss[0]), float(loss[-1])]}
    steps = max(3, min(args.steps, 20))
    guesses = (("plain", merc.WARM_PLAIN), ("learned", merc.WARM_MLP), ("series", merc.WARM_SERIES))
    # the large single system with the learned drift: 8196 planetesimals +
    # 131072 test particles (the network is the one trained above)
    c4 = systems.planetesimal_disk()
    hard_test = systems.hard_drifts(seed=20261213)
    for name, sysm in (("embryo_disk", c1), ("sweep", c2), ("planetesimal_disk", c4), ("hard_drifts", hard_test)):
        res = {}
        states = {}
        for key, warm in guesses:
            gi = merc.Integrator(merc.default_params(dt=sysm.dt, hill_factor=sysm.hill_factor,
                                                     drift=merc.DRIFT_UNIVERSAL, warm_start=warm), device=local)
            gi.load_systems(sysm)
            if warm == merc.WARM_MLP:
                gi.mlp_set_weights(w)
            gi.step(2)
            gi.step(steps)
            st = gi.stats()
            solves = max(st.kepler_solves, 1)
            res[key] = {"mean_iterations": st.kepler_iterations / solves,
                        "simt_iterations": st.kepler_simt_iterations / solves,
                        "ms_per_step": st.last_step_ms / steps, "nonconverged": int(st.kepler_nonconverged)}
            states[key] = gi.state().pos
            gi.close()
        a = states["plain"].reshape(3, -1)
        for key in ("learned", "series"):
            b = states[key].reshape(3, -1)
            ok = np.isfinite(a).all(0) & np.isfinite(b).all(0)
            d = np.abs(a[:, ok] - b[:, ok]).max(0) / np.linalg.norm(a[:, ok], axis=0)
            res[key]["max_rel_pos_diff_vs_plain"] = float(d.max())
            res[key]["p999_rel_pos_diff_vs_plain"] = float(np.quantile(d, 0.999))
        res["iteration_cut"] = res["plain"]["mean_iterations"] / res["learned"]["mean_iterations"]
        res["simt_iteration_cut"] = res["plain"]["simt_iterations"] / res["learned"]["simt_iterations"]
        res["simt_iteration_cut_vs_series"] = res["series"]["simt_iterations"] / res["learned"]["simt_iterations"]
        out[name] = res
    return out


def run_ours(args, world, rank, local, dist):
    import merc

    sysm = workload()
    n = sysm.n_total
    kw = dict(dt=sysm.dt, hill_factor=sysm.hill_factor, drift=merc.DRIFT_UNIVERSAL)
    g = merc.Integrator(merc.default_params(**kw), device=local)
    g.load_systems(sysm)
    g.time_kicks(True)
    peak = merc.fp64_peak_tflops(local)
    g.step(args.warmup)
    # the timed region's start state, for the end-to-end replay below
    start = g.state()
    start_alag = g.a_lag()
    l0 = g.launch_count()
    clocks = ClockSampler(local)
    clocks.start()
    if dist is not None:
        dist.barrier()
    step_ms, kick_ms, kick_n = [], 0.0, 0
    S = args.batch
    for _ in range(args.steps):
        g.flush_l2(512 << 20)
        g.step(S)
        step_ms.append(g.stats().last_step_ms)
        km, kc = g.kick_ms()
        kick_ms += km * kc
        kick_n += kc
    if dist is not None:
        dist.barrier()
    ck = clocks.stop()
    launches = g.launch_count() - l0
    total_ms = max_over_ranks(dist, float(np.sum(step_ms)))
    value = sum_over_ranks(dist, float(n * S * args.steps)) / (total_ms / 1e3)
    kick_avg_ms = kick_ms / max(kick_n, 1)
    nm = int(sysm.n_massive[0])
    pairs_per_kick = nm * (nm - 1) + (n - nm) * nm
    achieved = FLOPS_PER_PAIR * pairs_per_kick / (kick_avg_ms * 1e-3) / 1e12
    traffic = load_traffic().get("kick_bytes_per_launch")
    st = g.stats()

    # end to end through the C ABI with host buffers: the timed region's K
    # calls again, from its start state and with the same L2 flush before each
    # call (untimed); each call uploads the state from pinned host memory
    # (set_state), steps, and reads the result back into pinned memory
    # (get_state), so the copies are the only difference from `value`
    try:
        import torch

        pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()  # noqa: E731
        pos_h, vel_h, alag_h = pin(start.pos), pin(start.vel), pin(start_alag)
        flags_h = pin(start.flags)
        pinned = True
    except Exception:
        pos_h, vel_h, alag_h, flags_h = start.pos.copy(), start.vel.copy(), start_alag.copy(), start.flags.copy()
        pinned = False
    import merc as _m

    out_h = _m.State(pos_h, vel_h, flags_h)
    e2e_s = 0.0
    for _ in range(args.steps):
        g.flush_l2(512 << 20)
        t0 = time.perf_counter()
        g.set_state(pos_h, vel_h, alag_h)
        g.step(S)
        g.state(out=out_h)
        e2e_s += time.perf_counter() - t0
    e2e_s = max_over_ranks(dist, e2e_s)
    e2e_value = sum_over_ranks(dist, float(n * S * args.steps)) / e2e_s

    # the encounter sub-step (the largest share of the step at this encounter
    # density): a few more timed calls with events around its kernel
    g.time_kicks(False)
    g.time_encounter(True)
    enc_ms, enc_n, ce0, enc_calls = 0.0, 0, g.stats().ce_body_steps, 3
    for _ in range(enc_calls):
        g.flush_l2(512 << 20)
        g.step(S)
        em, ec = g.encounter_ms()
        enc_ms += em * ec
        enc_n += ec
    enc_avg_ms = enc_ms / max(enc_n, 1)
    ce_per_step = (g.stats().ce_body_steps - ce0) / (enc_calls * S)
    enc_pairs = ce_per_step * 7 * nm  # 7 evaluations of the sub-step, each over every massive source
    enc_achieved = FLOPS_PER_PAIR * enc_pairs / (enc_avg_ms * 1e-3) / 1e12
    g.time_encounter(False)

    # element-drift (reference-compat, bitwise-checked) path, same workload
    compat = None
    if not args.skip_compat:
        gc = merc.Integrator(merc.default_params(dt=sysm.dt, hill_factor=sysm.hill_factor,
                                                 drift=merc.DRIFT_ELEMENTS))
        gc.load_systems(sysm)
        gc.step(2)
        cs = max(2, min(args.steps, 10))
        gc.step(cs)
        compat = {"value": n * cs / (gc.stats().last_step_ms / 1e3), "steps": cs, "drift": "elements",
                  "note": "the reference's algorithm on the GPU, bit for bit with the oracle; compare with "
                          "cpu_baseline (the same algorithm on the host cores)"}
        gc.close()
    g.close()
    sweep = None if args.skip_sweep else sweep_section(merc, args, local, dist, world, rank)
    p9 = None if args.skip_p9 else p9_section(merc, args, local, dist, world, rank)
    planet = None if args.skip_planetesimal else planetesimal_section(merc, args, local, dist, world, rank, peak)
    if sweep:
        sweep["kick_fp64_frac_algorithmic"] = FLOPS_PER_PAIR * sweep["batched_pairs_per_s"] / 1e12 / peak
        sweep["kick_fp64_frac_note"] = ("pair work only (27 flops per pair over the measured FP64 FMA peak); the "
                                        "drift's Stumpff/Newton work, the larger share of this workload, is not "
                                        "counted")
    warm = None if args.skip_warm else warm_start_section(merc, args, local)

    if rank != 0:
        return
    cpu = cpu_ref = None
    if not args.skip_cpu:
        # the reference's step (element drift) as the baseline; the universal
        # drift on the same cores beside it
        cpu = cpu_rate(sysm, dict(kw, drift=0), sample_s=12.0)
        cpu_ref = cpu_rate(sysm, kw, sample_s=8.0)
        if compat:
            compat["gpu_over_cpu_same_algorithm"] = compat["value"] / cpu["value"]
        if sweep:
            sweep.update(sweep_cpu(sweep))
        if p9:
            p9.update(p9_cpu())
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded embryo disk)",
        "config": {"workload": sysm.label, "bodies": n, "n_massive": nm, "dt": sysm.dt, "drift": "universal",
                   "hill_factor": sysm.hill_factor, "batch": S,
                   "step": f"one merc_step call of {S} integrator steps",
                   "l2": "flushed (512 MB write) between timed steps",
                   "parallelism": f"replicas x{world}"},
        "roofline": {"bound": "fp64", "kernel": "k_sym (far-field pair sweep of the kick)", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "peak_source": "measured FP64 FMA loop on this GPU (merc_diag_fp64_peak)",
                     "kick_ms": kick_avg_ms, "kick_launches": kick_n, "pairs_per_launch": pairs_per_kick,
                     "flops_per_pair": FLOPS_PER_PAIR,
                     # utilisation beside the algorithmic figure: the kernel
                     # evaluates each unordered pair once in 22 FP64
                     # instructions (both directions), against the measured
                     # FP64 instruction rate (peak / 2: an FMA is 2 flops)
                     "fp64_instructions_per_unordered_pair": 22,
                     "issue_frac": 22 * (nm * (nm - 1) / 2) / (kick_avg_ms * 1e-3) / (peak * 1e12 / 2)},
        "roofline_encounter": {"bound": "fp64", "kernel": "k_encounter_tasks (encounter sub-step)",
                               "achieved": enc_achieved, "peak": peak, "unit": "TFLOP/s",
                               "frac": enc_achieved / peak, "encounter_ms": enc_avg_ms, "launches": enc_n,
                               "encounter_bodies_per_step": ce_per_step, "pairs_per_launch": enc_pairs,
                               "flops_per_pair": FLOPS_PER_PAIR,
                               "fp64_instructions_per_pair": 18,
                               "issue_frac": 18 * enc_pairs / (enc_avg_ms * 1e-3) / (peak * 1e12 / 2)},
        "cpu_baseline": cpu,
        "cpu_universal_drift": cpu_ref,
        "e2e": {"value": e2e_value, "unit": UNIT,
                "h2d_bytes_per_step": int(pos_h.nbytes + vel_h.nbytes + alag_h.nbytes),
                "d2h_bytes_per_step": int(pos_h.nbytes + vel_h.nbytes + flags_h.nbytes), "steps": args.steps,
                "pinned": pinned, "start": "the timed region's start state, same L2 flush before each call"},
        "pairs_per_s": value * 2 * (nm - 1) if n == nm else None,
        "gpu_launches": int(launches),
        "clocks": ck,
        "close_encounter_body_steps": int(st.ce_body_steps),
        "kepler_mean_iterations": (st.kepler_iterations / st.kepler_solves) if st.kepler_solves else None,
        "compat_elements_path": compat,
        "sweep": sweep,
        "p9_reference_workload": p9,
        "planetesimal_disk": planet,
        "learned_warm_start": warm,
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--batch", type=int, default=64, help="integrator steps per bench step (one merc_step call)")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-compat", action="store_true")
    ap.add_argument("--skip-sweep", action="store_true")
    ap.add_argument("--skip-warm", action="store_true")
    ap.add_argument("--skip-p9", action="store_true")
    ap.add_argument("--skip-planetesimal", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        # the CPU reference runs on rank 0 only; other ranks have no work
        if int(os.environ.get("RANK", "0")) == 0:
            run_reference(args, int(os.environ.get("WORLD_SIZE", "1")), 0, None)
        return
    world, rank, local, dist = dist_setup()
    if True:
        run_ours(args, world, rank, local, dist)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
