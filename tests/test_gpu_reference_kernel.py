"""The element path against the reference's own kernel running on the GPU.

oracle/refgpu/prepare.py copies the reference's mercurius_solver with its two
compile fixes (and a barrier before the kernel exits) into baseline/_ref/refgpu,
build() compiles it for sm_103a, and oracle/refgpu/refgpu.py launches it the way
the reference's host program does (clusters of 16 blocks of N/16 threads, four
sweeps per launch).  The reference evaluates sin, cos, atan2, acos, cbrt, ...
with CUDA's library and this library with its own, so the two element paths
agree to the element drift's amplification of a few ulps (measured: 4.5e-12 of
the position after 100 steps of the padded outer solar system, 3.2e-10 for the
Planet Nine systems; the oracle with the host's C library sits at the same
distance).  Skipped where the patched copy was not prepared.
"""
import os
import sys

import pytest

pytestmark = pytest.mark.gpu

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle", "refgpu"))
import refgpu  # noqa: E402

needs_ref = pytest.mark.skipif(not refgpu.available(), reason="the reference kernel was not prepared and built")


@needs_ref
@pytest.mark.parametrize("launches", [1, 2])
def test_element_path_matches_reference_kernel_outer(launches):
    """100 steps in one launch, and 2 launches of 50 steps (the batch boundary:
    the reference's epilogue writes elements and the next prologue reads them)."""
    batch, el = refgpu.outer_padded()
    r = refgpu.compare(batch, el, 100 // launches, 0.5, 1.0, 7, launches=launches)
    mx, med, nonfinite = r["ours_elements_vs_reference_gpu"]
    omx, omed, _ = r["oracle_host_libm_vs_reference_gpu"]
    assert nonfinite == 0
    assert mx <= 1e-9 and med <= 1e-12, r
    # no further from the reference than the oracle with the host's C library
    assert mx <= 10 * max(omx, 1e-12), r


@needs_ref
def test_element_path_matches_reference_kernel_p9():
    batch, el = refgpu.p9()
    r = refgpu.compare(batch, el, 100, 0.8219, 1.0, 640)
    mx, med, nonfinite = r["ours_elements_vs_reference_gpu"]
    assert nonfinite == 0
    assert mx <= 1e-8 and med <= 1e-12, r
