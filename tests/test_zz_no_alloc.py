"""The allocation-free budget entry point (obgc_tracer_budget_static) against the context one.

obgc_tracer_budget_static serves callers that cannot allocate device memory: a host whose device
memory belongs to another allocator's pool (CUDA.jl, PyTorch's caching allocator), or one working
under a fixed device-memory budget.  Its scratch is a static device array, so this test checks two
calls in a row (the second must not see the first one's partial sums) against
obgc_tracer_budget, which reduces into a buffer its context allocated.  The file sorts last so a
run that stops at the first failure has run every other test before it.
"""
import ctypes as C

import numpy as np
import pytest

import obgc
from obgc import _abi as A
from gpuhelp import cuda

pytestmark = pytest.mark.gpu


def static_budget(model, names, scales):
    lib = A.load()
    g = model.grid.c_grid()
    dt = A.F32 if model.precision == "f32" else A.F64
    ptrs = (C.c_void_p * len(names))(*[model.tracers[n].data_ptr() for n in names])
    sc = (C.c_double * len(names))(*scales)
    out = C.c_double(0.0)
    rc = lib.obgc_tracer_budget_static(C.byref(g), dt, len(names), ptrs, sc, C.byref(out),
                                       C.c_void_p(model._stream().value))
    return rc, out.value


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_static_budget_matches_context_budget_on_two_calls(precision):
    torch = cuda()
    g = obgc.RectilinearGrid((40, 24, 12), (4000.0, 2400.0, 120.0), dtype="f32" if precision == "f32" else "f64")
    bgc = obgc.LOBSTER(g, carbonate_system=obgc.CarbonateSystem())
    u, v, _ = obgc.random_streamfunction_velocity(g, rms=0.1, seed=5)
    model = obgc.NonhydrostaticModel(g, biogeochemistry=bgc, tracers=("T", "S"), velocities=(u, v, None),
                                     precision=precision)
    obgc.set_(model, **obgc.lobster_initial_conditions(g, seed=6))
    nitrogen, carbon = obgc.conserved_tracers(bgc)

    # first call: nitrogen group, same tolerance as the compensated-sum test of the context path
    rc, got = static_budget(model, nitrogen, [1.0] * len(nitrogen))
    assert rc == 0, A.load().obgc_last_error_message()
    ref = model.budget("nitrogen")
    assert abs(got - ref) <= 1e-15 * abs(ref)

    # second call in a row, on a different sum (carbon group after a step): no stale partials
    obgc.time_step(model, 300.0, nsteps=1)
    rc, got2 = static_budget(model, carbon["tracers"], carbon["scalefactors"])
    assert rc == 0, A.load().obgc_last_error_message()
    ref2 = model.budget("carbon")
    assert abs(got2 - ref2) <= 1e-15 * abs(ref2)
    assert got2 != got


def test_static_budget_grid_stride_at_the_block_cap():
    """128 x 128 x 16 cells is more than 4 blocks per SM x 256 threads: every block loops over
    several cells and the block count sits at its cap, on two calls in a row."""
    torch = cuda()
    g = obgc.RectilinearGrid((128, 128, 16), (25000.0, 25000.0, 160.0), dtype="f64")
    bgc = obgc.LOBSTER(g, carbonate_system=obgc.CarbonateSystem())
    u, v, _ = obgc.random_streamfunction_velocity(g, rms=0.1, seed=7)
    model = obgc.NonhydrostaticModel(g, biogeochemistry=bgc, tracers=("T", "S"), velocities=(u, v, None),
                                     precision="f64")
    obgc.set_(model, **obgc.lobster_initial_conditions(g, seed=8))
    nsm = torch.cuda.get_device_properties(0).multi_processor_count
    assert g.N > 4 * nsm * 256
    nitrogen, _ = obgc.conserved_tracers(bgc)
    for _ in range(2):
        rc, got = static_budget(model, nitrogen, [1.0] * len(nitrogen))
        assert rc == 0, A.load().obgc_last_error_message()
        ref = model.budget("nitrogen")
        assert abs(got - ref) <= 1e-15 * abs(ref)
        obgc.time_step(model, 300.0, nsteps=1)


def test_static_budget_rejects_too_many_fields():
    torch = cuda()
    g = obgc.RectilinearGrid((8, 8, 4), (1.0, 1.0, 4.0))
    fields = [torch.ones(g.shape, dtype=torch.float64, device="cuda") for _ in range(A.NUM_NAMED)]
    lib = A.load()
    n = 9   # OBGC_BUDGET_STATIC_MAX_FIELDS + 1
    ptrs = (C.c_void_p * n)(*[f.data_ptr() for f in fields[:n]])
    sc = (C.c_double * n)(*([1.0] * n))
    out = C.c_double(0.0)
    rc = lib.obgc_tracer_budget_static(C.byref(g.c_grid()), A.F64, n, ptrs, sc, C.byref(out), None)
    assert rc == 1
    assert "at most 8 fields" in lib.obgc_last_error_message().decode()
