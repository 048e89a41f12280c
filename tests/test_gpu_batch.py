"""Batched configuration: many independent problems in one persistent launch.

Problems follow the batched configuration's generator (d in {2,3,4}, SG level, deg in 2..4,
dense N(0,1/deg) 1-D operators, f ~ N(0,1)); the test keeps levels at 3..5 so the oracle and
the sequential launches stay quick.  The full draw (levels 3..7, 256 problems) is benchmarked.
"""
import numpy as np
import pytest

from cases import rel2
from oracle import asgard_oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def draw_problems(seed, count, lev_hi):
    import asgkron

    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        d = int(rng.choice([2, 3, 4]))
        lev = int(rng.integers(3, lev_hi + 1))
        deg = int(rng.integers(2, 5))
        table = asgkron.hash_table_sparse_nD([lev] * d, 8)
        n = deg * 2 ** lev
        mats = [[rng.normal(0.0, 1.0 / np.sqrt(deg), (n, n)) for _ in range(d)] for _ in range(d)]
        f = rng.standard_normal(table.num_elems * deg ** d)
        out.append((table.idx1d(), mats, deg, f))
    return out


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")


def test_batch_matches_single_plans_and_oracle(dev):
    import asgkron
    from asgkron.batch import Batch

    probs = draw_problems(3, 24, 5)
    plans = [asgkron.Plan.create(m, idx, deg, structure="detect") for idx, m, deg, _ in probs]
    fs = [torch.from_numpy(f).to(dev) for *_, f in probs]
    ys = [torch.empty_like(f) for f in fs]
    b = Batch(plans)
    b.set_io(fs, ys)
    b.apply()
    torch.cuda.synchronize()
    for k, ((idx, mats, deg, f), p) in enumerate(zip(probs, plans)):
        single = p.apply(fs[k])
        torch.cuda.synchronize()
        assert torch.equal(ys[k], single), k  # same algorithm, same order: bitwise
        N = idx.shape[0]
        rows = np.arange(0, N, max(1, N // 4))
        want = O.apply_A_rows(mats, idx.astype(np.int64), deg, f, rows=rows)
        got = ys[k].cpu().numpy().reshape(N, -1)[rows].ravel()
        assert rel2(got, want) <= 1e-12, k
    # FP32 batch within 1e-6 of FP64; tuned and graph-captured replays agree bitwise
    fs32 = [f.float() for f in fs]
    ys32 = [torch.empty_like(f) for f in fs32]
    b32 = Batch(plans)
    b32.set_io(fs32, ys32)
    ms = b32.tune()
    assert ms > 0
    b32.apply()
    torch.cuda.synchronize()
    first = [y.clone() for y in ys32]
    for k in range(len(probs)):
        assert rel2(ys32[k].double().cpu().numpy(), ys[k].cpu().numpy()) <= 1e-6, k
    b32.capture()
    for y in ys32:
        y.zero_()
    b32.graph.replay()
    torch.cuda.synchronize()
    for a, c in zip(ys32, first):
        assert torch.equal(a, c)
    info = b32.info()
    assert info["warps_per_cta"] in (4, 8) and info["rows_per_item"] in (1, 2, 4)


@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_batch_launch_shapes_bitwise(dev, dtype):
    """Every (warps per CTA, rows per item) shape equals the single-plan launches bitwise: a
    warp computes up to four rows of a small-block problem side by side (deg 1..4, d 2..4,
    row counts not multiples of the rows per item), each with the single-row arithmetic."""
    import asgkron
    from asgkron.batch import Batch

    rng = np.random.default_rng(11)
    plans, fs = [], []
    for deg in (1, 2, 3, 4):
        for d in (2, 3, 4):
            lev = 3
            table = asgkron.hash_table_sparse_nD([lev] * d, 8)
            n = deg * 2 ** lev
            mats = [[rng.normal(0.0, 1.0 / np.sqrt(deg), (n, n)) for _ in range(d)] for _ in range(d)]
            plans.append(asgkron.Plan.create(mats, table.idx1d(), deg, structure="detect"))
            fs.append(torch.from_numpy(rng.standard_normal(table.num_elems * deg ** d)).to(dev, getattr(torch, dtype)))
    singles = [p.apply(f) for p, f in zip(plans, fs)]
    ys = [torch.empty_like(f) for f in fs]
    b = Batch(plans)
    b.set_io(fs, ys)
    for wpb, rpi in ((4, 1), (8, 2), (4, 4)):
        b.configure(wpb, rpi)
        for y in ys:
            y.fill_(float("nan"))
        b.apply()
        torch.cuda.synchronize()
        assert b.info()["rows_per_item"] == rpi
        for k, (y, want) in enumerate(zip(ys, singles)):
            assert torch.equal(y, want), (wpb, rpi, k)


def test_batch_configure_rejects_bad_shapes(dev):
    import asgkron
    from asgkron._lib import AsgError
    from asgkron.batch import Batch
    from cases import problem

    _, _, idx, mats = problem("continuity2", 3, 2)
    b = Batch([asgkron.Plan.create(mats, idx, 2)])
    with pytest.raises(AsgError, match="warps_per_cta=6"):
        b.configure(6, 1)
    with pytest.raises(AsgError, match="rows_per_item=3"):
        b.configure(4, 3)


def test_batch_rejects_large_blocks(dev):
    import asgkron
    from asgkron._lib import AsgError
    from asgkron.batch import Batch
    from cases import problem

    _, _, idx, mats = problem("continuity6", 2, 4)  # 4^6 = 4096 > 256
    p = asgkron.Plan.create(mats, idx, 4)
    with pytest.raises(AsgError, match="deg\\^d=4096"):
        Batch([p])


def test_batch_levels_6_7_vs_oracle(dev):
    """The batched configuration's own draw (seed 3, levels 3..7): its first level-6 and first
    level-7 problem in one FP32 persistent launch, sampled rows against the C restatement of
    the reference loop (apply_A.m:102-236, all pairs, FP64)."""
    import asgkron
    from asgkron.batch import Batch
    from oracle import cref

    rng = np.random.default_rng(3)
    picked = {}
    for _ in range(256):  # the generator's order: d, level, degree, operators, f
        d = int(rng.choice([2, 3, 4]))
        lev = int(rng.integers(3, 8))
        deg = int(rng.integers(2, 5))
        table = asgkron.hash_table_sparse_nD([lev] * d, 8)
        n = deg * 2 ** lev
        mats = [[rng.normal(0.0, 1.0 / np.sqrt(deg), (n, n)) for _ in range(d)] for _ in range(d)]
        f = rng.standard_normal(table.num_elems * deg ** d)
        if lev in (6, 7) and lev not in picked:
            picked[lev] = (table.idx1d(), mats, deg, f)
        if len(picked) == 2:
            break
    assert sorted(picked) == [6, 7]
    probs = [picked[6], picked[7]]
    plans = [asgkron.Plan.create(m, idx, deg, structure="none") for idx, m, deg, _ in probs]
    fs = [torch.from_numpy(f).to(dev).float() for *_, f in probs]
    ys = [torch.empty_like(f) for f in fs]
    b = Batch(plans)
    b.set_io(fs, ys)
    b.apply()
    torch.cuda.synchronize()
    for (idx, mats, deg, f), y in zip(probs, ys):
        N = idx.shape[0]
        rows = np.array([0, N // 3, N - 1], dtype=np.int32)
        want = cref.apply_rows(mats, idx, deg, f, rows=rows)
        got = y.double().cpu().numpy().reshape(N, -1)[rows].ravel()
        assert rel2(got, want) <= 1e-6, (N, deg)
    b.close()
    for p in plans:
        p.close()
