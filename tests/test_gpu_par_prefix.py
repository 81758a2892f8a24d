"""The TwoBand chlorophyll sums above each work item's segment come from a pre-pass kernel
(par_prefix_kernel) when the segments are two levels or longer, and from the work items themselves
for one-level segments.  Both sum the same terms in the same order from the surface down, so the
step is the same bit for bit whatever the segment length, and agrees with the oracle."""
import numpy as np
import pytest

import obgc
import oracle as O
from gpuhelp import cuda, rel_err

pytestmark = pytest.mark.gpu


def run(precision, TZ, staging=1, nsteps=3, shape=(40, 24, 20)):
    cuda()
    g = obgc.RectilinearGrid(shape, (4000.0, 2400.0, 200.0), dtype="f32" if precision == "f32" else "f64")
    bgc = obgc.LOBSTER(g, carbonate_system=obgc.CarbonateSystem())
    u, v, _ = obgc.random_streamfunction_velocity(g, rms=0.1, seed=4)
    model = obgc.NonhydrostaticModel(g, biogeochemistry=bgc, tracers=("T", "S"), velocities=(u, v, None),
                                     precision=precision)
    model.set_tiling(TZ)
    model.set_staging(staging)
    obgc.set_(model, **obgc.lobster_initial_conditions(g, seed=5))
    s0 = model.state_array().double().cpu().numpy()
    obgc.time_step(model, 300.0, nsteps=nsteps)
    return g, bgc, (u, v), model, s0, model.state_array().double().cpu().numpy()


@pytest.mark.parametrize("precision", ["f32", "mixed", "f64"])
def test_segment_length_does_not_change_the_step(precision):
    # 1 level: the items sum (10 pre-pass segments fit a 20-level grid); 3 and 8: the pre-pass
    _, _, _, _, _, ref = run(precision, 1)
    for TZ in (3, 8):
        _, _, _, model, _, got = run(precision, TZ)
        assert np.array_equal(got, ref), (TZ, max(rel_err(got[q], ref[q]) for q in range(got.shape[0])))
    assert model.last_timing()[2] > 0


def test_pre_pass_steps_match_the_oracle():
    g, bgc, vel, model, s0, got = run("f64", 4, nsteps=4)
    m = O.model3d(bgc.params, g.c_grid(), model.tracer_names)
    ref = np.ascontiguousarray(s0.copy())
    u, v = (x.double().cpu().numpy().ravel().copy() for x in vel)
    O.step3d(m, ref, u=u, v=v, t=0.0, dt=300.0, nsteps=4)
    assert max(rel_err(got[q], ref[q]) for q in range(got.shape[0])) < 1e-11


def test_pre_pass_with_cp_async_staging_and_graph_replay():
    _, _, _, _, _, ref = run("f32", 1, staging=0)
    _, _, _, _, _, got = run("f32", 5, staging=0)
    assert np.array_equal(got, ref)
    # the same steps from a CUDA graph
    cuda()
    g = obgc.RectilinearGrid((40, 24, 20), (4000.0, 2400.0, 200.0), dtype="f32")
    bgc = obgc.LOBSTER(g, carbonate_system=obgc.CarbonateSystem())
    u, v, _ = obgc.random_streamfunction_velocity(g, rms=0.1, seed=4)
    model = obgc.NonhydrostaticModel(g, biogeochemistry=bgc, tracers=("T", "S"), velocities=(u, v, None), precision="f32")
    model.set_tiling(5)
    model.set_staging(0)
    obgc.set_(model, **obgc.lobster_initial_conditions(g, seed=5))
    obgc.time_step(model, 300.0, nsteps=3, graph=True)
    assert np.array_equal(model.state_array().double().cpu().numpy(), ref)
