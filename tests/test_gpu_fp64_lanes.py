"""How the FP64 pipe charges a partially active warp instruction, the premise
of the kernels' branch-free FP64 code (the cubic spline's two pieces as one
operation sequence, the mirrored Riemann problems, sign flips on the integer
pipe): a warp whose FMA chains run on one lane takes about as long as one
whose 32 lanes run them, so an idle lane is not given back."""
import pytest

pytestmark = pytest.mark.gpu


def test_idle_lanes_are_not_reclaimed():
    from meshlesshydro_gb300 import build, runtime
    build.build()
    t32 = runtime.probe_fp64_lanes(32)
    t8 = runtime.probe_fp64_lanes(8)
    t1 = runtime.probe_fp64_lanes(1)
    assert t32 > 0 and t8 > 0 and t1 > 0
    # per-lane throughput with one active lane is far below the full warp's
    # (GB300: t1 ~ t8 ~ t32, i.e. 1/32 of it)
    assert t1 > t32 / 8
    assert t8 > t32 / 2
