"""GPU: batches of uneven BTA matrices (mixed float32/float64, with and
without arrowhead, several RHS) in one graph launch, against the oracle."""

import numpy as np
import pytest
import torch

import oracle
from serinv_gb300.batched import BatchPlan
from serinv_gb300.synthetic import generate

from _golden import rel_err

pytestmark = pytest.mark.gpu

TOL = {np.dtype(np.float64): 1e-12, np.dtype(np.float32): 1e-5}


def make_batch(count, seed=0):
    rng = np.random.default_rng(seed)
    mats = []
    for i in range(count):
        n = int(rng.integers(2, 12))
        b = int(rng.choice([8, 32, 40, 64]))
        a = int(rng.choice([0, 4, 16]))
        dt = np.float32 if i % 2 == 0 else np.float64
        mats.append(generate(n, b, a, 4, seed=i, dtype=dt))
    return mats


def oracle_run(m):
    r = m.copy()
    oracle.pobtaf(*r.arrays())
    L = [x.copy() for x in r.arrays()]
    x = r.B.copy()
    oracle.pobtas(*L, x, trans="N")
    oracle.pobtas(*L, x, trans="T")
    oracle.pobtasi(*r.arrays())
    return L, list(r.arrays()), x


@pytest.mark.parametrize("nstreams", [1, 4, 16])
def test_batch_against_oracle(nstreams):
    mats = make_batch(12, seed=nstreams)
    dev = [tuple(torch.from_numpy(x).cuda() for x in m.arrays()) for m in mats]
    rhs = [torch.from_numpy(m.B).cuda() for m in mats]
    plan = BatchPlan(dev, rhs, nstreams=nstreams)
    plan.run()
    torch.cuda.synchronize()
    assert torch.all(plan.info() == 0)
    for m, d, r in zip(mats, dev, rhs):
        L, X, x = oracle_run(m)
        tol = TOL[m.D.dtype]
        for got, ref in zip(d, X):
            if ref.size:
                assert rel_err(got.cpu().numpy(), ref) <= tol
        assert rel_err(r.cpu().numpy(), x) <= tol
    plan.close()


def test_batch_replay_is_idempotent_on_fresh_inputs():
    mats = make_batch(6, seed=7)
    src = [tuple(torch.from_numpy(x).cuda() for x in m.arrays()) for m in mats]
    dev = [tuple(x.clone() for x in s) for s in src]
    plan = BatchPlan(dev, None, ops=("pobtaf", "pobtasi"), nstreams=3)
    plan.run()
    first = [tuple(x.clone() for x in d) for d in dev]
    for d, s in zip(dev, src):
        for x, y in zip(d, s):
            x.copy_(y)
    plan.run()
    torch.cuda.synchronize()
    for d, f in zip(dev, first):
        for x, y in zip(d, f):
            assert torch.equal(x, y)
    plan.close()


def test_batch_reports_not_spd():
    mats = make_batch(4, seed=9)
    mats[2].D[0][0, 0] = -50.0
    dev = [tuple(torch.from_numpy(x).cuda() for x in m.arrays()) for m in mats]
    plan = BatchPlan(dev, None, ops=("pobtaf",), nstreams=2)
    plan.run()
    info = plan.info()
    assert int(info[2]) == 1
    assert int(info[0]) == 0 and int(info[1]) == 0 and int(info[3]) == 0
    plan.close()


def test_autotuner_picks_a_candidate(tmp_path, monkeypatch):
    import serinv_gb300.batched as bm
    monkeypatch.setattr(bm, "CACHE", str(tmp_path / "tune.json"))
    mats = make_batch(5, seed=11)
    dev = [tuple(torch.from_numpy(x).cuda() for x in m.arrays()) for m in mats]
    before = [tuple(x.clone() for x in d) for d in dev]
    ns = bm.autotune_nstreams(dev, None, ops=("pobtaf", "pobtasi"), candidates=(1, 2, 4))
    assert ns in (1, 2, 4)
    for d, b in zip(dev, before):  # tuning ran on scratch copies
        for x, y in zip(d, b):
            assert torch.equal(x, y)
    assert (tmp_path / "tune.json").exists()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_column_block_kernel_in_graph(precision):
    """Blocks of b > 64 run the cooperative column-block kernel inside the
    plan's graph (several side by side on part of the GPU)."""
    rng = np.random.default_rng(21)
    mats = []
    for i in range(8):
        n = int(rng.integers(2, 6))
        b = int(rng.choice([96, 128, 160]))
        a = int(rng.choice([0, 16]))
        dt = np.float32 if (i % 2 == 0 and precision == "fp64") else np.float64
        mats.append(generate(n, b, a, 4, seed=100 + i, dtype=dt))
    dev = [tuple(torch.from_numpy(x).cuda() for x in m.arrays()) for m in mats]
    rhs = [torch.from_numpy(m.B).cuda() for m in mats]
    plan = BatchPlan(dev, rhs, precisions=[precision] * len(mats), nstreams=4)
    plan.run()
    torch.cuda.synchronize()
    assert torch.all(plan.info() == 0)
    for m, d, r in zip(mats, dev, rhs):
        L, X, x = oracle_run(m)
        tol = TOL[m.D.dtype] if precision == "fp64" else 1e-9
        for got, ref in zip(d, X):
            if ref.size:
                assert rel_err(got.cpu().numpy(), ref) <= tol
        assert rel_err(r.cpu().numpy(), x) <= tol
    plan.close()


def test_batch_with_complex_matrices():
    """complex128 / complex64 matrices (through the real embedding) beside
    real ones in one plan."""
    rng = np.random.default_rng(5)
    mats = []
    for i in range(6):
        n = int(rng.integers(2, 6))
        b = int(rng.choice([8, 40, 96]))
        a = int(rng.choice([0, 4]))
        dt = [np.complex128, np.complex64, np.float64][i % 3]
        mats.append(generate(n, b, a, 2, seed=200 + i, dtype=dt))
    dev = [tuple(torch.from_numpy(x).cuda() for x in m.arrays()) for m in mats]
    rhs = [torch.from_numpy(m.B).cuda() for m in mats]
    plan = BatchPlan(dev, rhs, nstreams=3)
    plan.run()
    torch.cuda.synchronize()
    assert torch.all(plan.info() == 0)
    tol = {np.dtype(np.complex128): 1e-12, np.dtype(np.complex64): 1e-5, np.dtype(np.float64): 1e-12}
    for m, d, r in zip(mats, dev, rhs):
        L, X, x = oracle_run(m)
        for got, ref in zip(d, X):
            if ref.size:
                assert rel_err(got.cpu().numpy(), ref) <= tol[m.D.dtype]
        assert rel_err(r.cpu().numpy(), x) <= tol[m.D.dtype]
    plan.close()


def test_plan_panel_cta_counts_agree_with_the_oracle():
    """The column-block CTA count is a schedule choice only: 18, 32 and a
    count too small for the kernel's roles (the launch-based tile sweep)
    give the oracle's results."""
    rng = np.random.default_rng(33)
    mats = []
    for i in range(4):
        n = int(rng.integers(3, 7))
        b = int(rng.choice([96, 128]))
        mats.append(generate(n, b, 8, 2, seed=400 + i, dtype=np.float64))
    refs = [oracle_run(m) for m in mats]
    for panel, split in ((18, False), (32, True), (4, False)):
        dev = [tuple(torch.from_numpy(x.copy()).cuda() for x in m.arrays()) for m in mats]
        rhs = [torch.from_numpy(m.B.copy()).cuda() for m in mats]
        plan = BatchPlan(dev, rhs, nstreams=2, panel_ctas=panel, tc_ksplit=split)
        plan.run()
        torch.cuda.synchronize()
        assert torch.all(plan.info() == 0)
        for (L, X, x), d, r in zip(refs, dev, rhs):
            for got, ref in zip(d, X):
                if ref.size:
                    assert rel_err(got.cpu().numpy(), ref) <= 1e-12, panel
            assert rel_err(r.cpu().numpy(), x) <= 1e-12, panel
        plan.close()


def test_autotuner_returns_streams_and_panel_ctas(tmp_path, monkeypatch):
    import serinv_gb300.batched as bm
    monkeypatch.setattr(bm, "CACHE", str(tmp_path / "tune.json"))
    mats = make_batch(4, seed=12)
    dev = [tuple(torch.from_numpy(x).cuda() for x in m.arrays()) for m in mats]
    ns, panel, split = bm.autotune(dev, None, ops=("pobtaf", "pobtasi"), candidates=(1, 2),
                                   panel_candidates=(18, 24))
    assert ns in (1, 2) and panel in (0, 18) and split in (True, False)
    assert bm.autotune(dev, None, ops=("pobtaf", "pobtasi")) == (ns, panel, split)  # cached
