"""Integrate one of the benchmark workloads for a number of steps.

    python p9-integrator_gb300/run_workload.py --workload embryo|sweep|outer|planetesimal|p9
           [--steps N] [--warmup W] [--drift universal|elements] [--systems S]

Prints one line with device time per step.  The profiling commands in
profiles/ run it under ncu, so that one kernel of one workload can be captured
without the rest of bench.py.
"""
import argparse
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

import merc  # noqa: E402
import systems  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="embryo", choices=["embryo", "sweep", "outer", "planetesimal", "p9"])
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=2)
    ap.add_argument("--drift", default="universal", choices=["universal", "elements"])
    ap.add_argument("--systems", type=int, default=4096, help="sweep: number of systems (p9: sweeps, default 32)")
    ap.add_argument("--test-particles", type=int, default=131072, help="planetesimal: test particles")
    a = ap.parse_args()
    if a.workload == "embryo":
        s = systems.embryo_disk()
    elif a.workload == "sweep":
        s = systems.sweep(n_systems=a.systems)
    elif a.workload == "outer":
        s = systems.outer_solar_system()
    elif a.workload == "p9":
        s = systems.p9_sweep(n_sweeps=a.systems if a.systems != 4096 else 32)
    else:
        s = systems.planetesimal_disk(n_test=a.test_particles)
    drift = merc.DRIFT_UNIVERSAL if a.drift == "universal" else merc.DRIFT_ELEMENTS
    g = merc.Integrator(merc.default_params(dt=s.dt, hill_factor=s.hill_factor, drift=drift))
    g.load_systems(s)
    g.step(a.warmup)
    g.step(a.steps)
    st = g.stats()
    print(f"{a.workload}: {s.n_total} bodies, {a.steps} steps, {st.last_step_ms / a.steps:.4f} ms/step, "
          f"{s.n_total * a.steps / (st.last_step_ms / 1e3):.4g} body-steps/s, encounters {st.ce_body_steps}")
    g.close()


if __name__ == "__main__":
    main()
