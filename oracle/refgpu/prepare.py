"""Prepare the reference's own CUDA kernel for GB300 (TEST INFRASTRUCTURE).

Copies the reference's src/sim.cuh, src/simutils.cuh, src/constants.cuh and
src/json.hpp from the reference checkout (MERC_REF_DIR, else the oracle build
recipe's default) into baseline/_ref/refgpu/ (git-ignored; it travels to the
GPU host, where the reference checkout does not exist) and applies these
textual patches, each of which must match exactly once:

  1. sim.cuh:147 calls an undefined magnitude(): r_mag = sqrt(|r|^2)
     (the compile fix the reference needs; same value as norm3d up to rounding).
  2. sim.cuh:173 calls fetch_r_crit with four arguments, one of them the
     undeclared `masses`; the function takes (mapped_block, index)
     (sim.cuh:133-135): the call becomes fetch_r_crit(mapped_block, idx_other).
  3. constants.cuh: BATCH_SIZE (steps per kernel launch, 1e6) becomes a value
     set at run time, so one launch can run 100 steps for a parity check.
  4. sim.cuh, end of mercurius_solver: a cluster.sync() after the epilogue's
     democratic-heliocentric conversion.  Every block reads block 0's shared
     memory there (sim.cuh:748) and nothing stops block 0 from exiting first;
     reading the shared memory of a block that has exited is undefined.  The
     added barrier is reached by every thread of the cluster once and changes
     no result.

Nothing else is changed.  build() then compiles refgpu_driver.cu (this
folder) against the patched copy for sm_103a, with the reference's own flags
(-O3, default contraction).

    python oracle/refgpu/prepare.py        # here, where the reference exists
"""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(ROOT, "baseline", "_ref", "refgpu")
FILES = ["sim.cuh", "simutils.cuh", "constants.cuh", "json.hpp"]

PATCHES = [
    ("sim.cuh", "  double r_mag = magnitude(r);\n", "  double r_mag = sqrt(magnitude_squared(r));\n"),
    ("sim.cuh", "fetch_r_crit(current_coords, masses, idx_other, dt);",
     "fetch_r_crit(mapped_block, idx_other);"),
    ("constants.cuh", "#define BATCH_SIZE 1000000\n",
     "__device__ long merc_ref_batch_steps_d = 1000000;\n"
     "static long merc_ref_batch_steps_h = 1000000;\n"
     "__host__ __device__ inline long merc_ref_batch_steps() {\n"
     "#ifdef __CUDA_ARCH__\n  return merc_ref_batch_steps_d;\n#else\n  return merc_ref_batch_steps_h;\n#endif\n}\n"
     "#define BATCH_SIZE merc_ref_batch_steps()\n"),
    ("sim.cuh",
     "  velocities[idx] = democratic_heliocentric_conversion((PosVel){.pos = positions[idx], .vel = velocities[idx]}, "
     "num_massive_bodies, &mapped_block, true);\n",
     "  velocities[idx] = democratic_heliocentric_conversion((PosVel){.pos = positions[idx], .vel = velocities[idx]}, "
     "num_massive_bodies, &mapped_block, true);\n  cluster.sync();\n"),
]


def main():
    sys.path.insert(0, os.path.dirname(HERE))
    from oracle import ref_dir

    ref = ref_dir()
    if ref is None:
        print("reference checkout not present: nothing prepared")
        return 1
    os.makedirs(OUT, exist_ok=True)
    text = {}
    for f in FILES:
        with open(os.path.join(ref, "src", f)) as fh:
            text[f] = fh.read()
    for f, old, new in PATCHES:
        n = text[f].count(old)
        if n != 1:
            raise SystemExit(f"patch for {f} matched {n} times (expected 1): {old[:60]!r}")
        text[f] = text[f].replace(old, new)
    for f in FILES:
        with open(os.path.join(OUT, f), "w") as fh:
            fh.write(text[f])
    print(f"patched reference kernel in {OUT}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
