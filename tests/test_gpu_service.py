"""The continuous-batching column service: every run's result is bit-for-bit the result of the same
run stepped alone, while runs join and leave the device around it; admission by the HBM budget;
latency statistics; and bounded waits."""
import time

import numpy as np
import pytest

import obgc
from gpuhelp import cuda

pytestmark = pytest.mark.gpu


def requests(n, seed, days=(0.1, 0.6)):
    rng = np.random.default_rng(seed)
    return [obgc.lobster_column_request(rng, levels=(8, 256), days=days) for _ in range(n)]


def alone(bgc, r, precision, co2=None):
    eng = obgc.ColumnEngine(bgc, precision=precision, max_columns=2, arena_cells=r["init"].shape[1] + 1,
                            co2_exchange=co2)
    s = eng.add(r["init"], r["kappa"], r["dz"], r["dt"], r["nsteps"], surface_PAR=r["surface_PAR"], mu0=r["mu0"],
                pulse_step=r["pulse_step"], pulse_k=r["pulse_k"], pulse_amount=r["pulse_amount"], T=r["T"], S=r["S"])
    while eng.remaining(s):
        eng.advance(97)
    out = eng.read(s)
    eng.close()
    return out


@pytest.mark.parametrize("precision,with_co2", [("f32", False), ("mixed", False), ("f32", True)])
def test_each_result_is_the_same_alone_and_in_the_mix(precision, with_co2):
    cuda()
    bgc = obgc.LOBSTER(None, carbonate_system=obgc.CarbonateSystem())
    co2 = obgc.CarbonDioxideGasExchangeBoundaryCondition(wind_speed=7.0) if with_co2 else None
    reqs = requests(30, seed=17)
    svc = obgc.ColumnService(bgc, precision=precision, max_columns=64, arena_cells=64 * 260, chunk_steps=16,
                             co2_exchange=co2)
    ids = []
    for wave in range(3):                       # later waves arrive while earlier runs are on the GPU
        for r in reqs[wave * 10:(wave + 1) * 10]:
            ids.append(svc.submit_request(r))
        time.sleep(0.02)
    results = [svc.wait(i, timeout=300) for i in ids]
    st = svc.stats()
    svc.close()
    assert st["completed"] == len(reqs) and st["launches"] > 0
    for r, (got, lat) in zip(reqs, results):
        assert lat > 0
        assert np.array_equal(got, alone(bgc, r, precision, co2))


def test_admission_waits_for_the_hbm_budget():
    cuda()
    bgc = obgc.NPZD(None)
    cols = obgc.npzd_column_ensemble(12, seed=5, levels=(100, 250), nsteps=40)
    svc = obgc.ColumnService(bgc, precision="f32", max_columns=64, arena_cells=520, chunk_steps=8)   # ~2-4 runs fit
    ids = [svc.submit_request(c) for c in cols]
    svc.drain(timeout=300)
    st = svc.stats()
    outs = [svc.wait(i)[0] for i in ids]
    svc.close()
    assert st["completed"] == 12 and st["admitted"] == 12
    for c, o in zip(cols, outs):
        assert o.shape == c["init"].shape and np.all(np.isfinite(o))
        assert np.array_equal(o, alone_npzd(bgc, c))


def alone_npzd(bgc, c):
    eng = obgc.ColumnEngine(bgc, precision="f32", max_columns=2, arena_cells=c["init"].shape[1] + 1)
    s = eng.add(c["init"], c["kappa"], c["dz"], c["dt"], c["nsteps"], surface_PAR=c["surface_PAR"], mu0=c["mu0"])
    eng.advance(c["nsteps"])
    out = eng.read(s)
    eng.close()
    return out


def test_latency_statistics_and_bounded_waits():
    cuda()
    bgc = obgc.NPZD(None)
    cols = obgc.npzd_column_ensemble(40, seed=8, levels=(16, 128), nsteps=64)
    svc = obgc.ColumnService(bgc, precision="f32", max_columns=128, arena_cells=128 * 130, chunk_steps=16)
    long_run = dict(cols[0], nsteps=200000)
    lid = svc.submit_request(long_run)
    with pytest.raises(obgc._abi.ObgcError) as ei:
        svc.wait(lid, timeout=0.05)                # bounded host-side wait on a run still in progress
    assert ei.value.status == 9                    # OBGC_ERR_TIMEOUT
    for c in cols:
        svc.submit_request(c)
    t0 = time.time()
    while svc.stats()["completed"] < len(cols) and time.time() - t0 < 300:
        time.sleep(0.01)
    st = svc.stats()
    assert st["completed"] >= len(cols)
    assert 0 < st["p50_ms"] <= st["p99_ms"] <= st["max_ms"]
    with pytest.raises(obgc._abi.ObgcError):
        svc.wait(123456789, timeout=0.01)          # unknown request
    svc.close()                                    # drops the long run after the chunk in flight
