"""The autotuner (l2c_gpu_autotune): per call shape it picks among launch
choices that never change results, so a tuned plan gives the untuned plan's
bits; its choices persist in the L2C_AUTOTUNE_CACHE file and are read back by
later plans of the same device, N, maxs and form; L2C_AUTOTUNE=1 tunes each new
shape on its first call."""
import numpy as np
import pytest

from tests.golden.cases import make_input

pytestmark = pytest.mark.gpu

SHAPES = [  # (N, maxs, count, lagrange, mixed)
    (65536, 64, 1, 0, False),
    (1024, 64, 64, 0, False),
    (4096, 36, 8, 1, False),
    (16384, 16, 16, 0, True),
]


def run(plan, x, count, N):
    outs = []
    for d in (0, 1):
        out = np.zeros_like(x)
        plan.execute_batched(x, out, d, count, N, 1)
        outs.append(out)
    return outs


@pytest.mark.parametrize("N,maxs,count,lagrange,mixed", SHAPES)
def test_tuned_calls_same_bits(lib, monkeypatch, N, maxs, count, lagrange, mixed):
    monkeypatch.delenv("L2C_AUTOTUNE", raising=False)
    monkeypatch.delenv("L2C_AUTOTUNE_CACHE", raising=False)
    x = np.ascontiguousarray(make_input(N * count, "gauss", N + count).reshape(count, N))
    want = run(lib.Plan(N, maxs, lagrange=lagrange, mixed=mixed), x, count, N)
    p = lib.Plan(N, maxs, lagrange=lagrange, mixed=mixed)
    for d in (0, 1):
        assert p.tuned_config(d, count, N, 1)[0] == "default"
        ms = p.autotune(d, count, N, 1)
        src, text, ms_tuned, ms_default = p.tuned_config(d, count, N, 1)
        assert src == "tuned" and ms == ms_tuned and 0 < ms_tuned <= ms_default, text
        assert "overlap=" in text and "near_vb=" in text and "near_table=" in text
    for _ in range(2):  # capture, then replay, under the tuned choices
        got = run(p, x, count, N)
        for d in (0, 1):
            assert np.array_equal(got[d], want[d]), d
    # another shape on the same plan keeps the plan's own choices
    assert p.tuned_config(0, 2, N, 1)[0] == "default"


def test_cache_round_trip(lib, monkeypatch, tmp_path):
    cache = tmp_path / "tune.txt"
    cache.write_text("not a cache line\nl2c-tune-1|x|1|2\n")
    monkeypatch.setenv("L2C_AUTOTUNE_CACHE", str(cache))
    monkeypatch.delenv("L2C_AUTOTUNE", raising=False)
    N, count = 2048, 8
    p = lib.Plan(N, 64)
    p.autotune(0, count, N, 1)
    src, text, ms, _ = p.tuned_config(0, count, N, 1)
    lines = [l for l in cache.read_text().splitlines() if l.startswith("l2c-tune-")]
    assert src == "tuned" and len(lines) == 2  # the malformed one and ours
    q = lib.Plan(N, 64)  # same device, N, maxs and form: read back
    src2, text2, ms2, _ = q.tuned_config(0, count, N, 1)
    assert (src2, text2) == ("cache", text) and abs(ms2 - ms) < 1e-5
    assert q.tuned_config(1, count, N, 1)[0] == "default"  # other direction
    assert lib.Plan(N, 32).tuned_config(0, count, N, 1)[0] == "default"  # other maxs
    assert lib.Plan(N, 64, mixed=True).tuned_config(0, count, N, 1)[0] == "default"
    x = np.ascontiguousarray(make_input(N * count, "sign", 5).reshape(count, N))
    a, b = np.zeros_like(x), np.zeros_like(x)
    q.execute_batched(x, a, 0, count, N, 1)
    monkeypatch.delenv("L2C_AUTOTUNE_CACHE")
    lib.Plan(N, 64).execute_batched(x, b, 0, count, N, 1)
    assert np.array_equal(a, b)


def test_tunes_on_first_call(lib, monkeypatch):
    monkeypatch.delenv("L2C_AUTOTUNE_CACHE", raising=False)
    N, count = 4096, 4
    x = np.ascontiguousarray(make_input(N * count, "uniform", 9).reshape(count, N))
    monkeypatch.setenv("L2C_AUTOTUNE", "0")
    want = run(lib.Plan(N, 64), x, count, N)
    monkeypatch.setenv("L2C_AUTOTUNE", "1")
    p = lib.Plan(N, 64)
    assert p.tuned_config(0, count, N, 1)[0] == "default"
    got = run(p, x, count, N)
    for d in (0, 1):
        assert p.tuned_config(d, count, N, 1)[0] == "tuned"
        assert np.array_equal(got[d], want[d])


def test_autotune_rejects_bad_shapes(lib, monkeypatch):
    monkeypatch.delenv("L2C_AUTOTUNE_CACHE", raising=False)
    p = lib.Plan(1024, 64, direction=0)
    with pytest.raises(lib.L2CError, match="not planned"):
        p.autotune(1, 1, 0, 1)
    with pytest.raises(lib.L2CError, match="count"):
        p.autotune(0, 0, 0, 1)
    with pytest.raises(lib.L2CError, match="dist"):
        p.autotune(0, 4, 0, 1)


def test_ragged_overlap_and_tuning_same_bits(lib, monkeypatch):
    """Ragged lists: the band and the direct-method vectors beside the
    far-field chain or not, the chain's priority, and the tuned choice give
    the same bits."""
    monkeypatch.delenv("L2C_AUTOTUNE", raising=False)
    rng = np.random.default_rng(8)
    Ns = [int(n) for n in np.exp(rng.uniform(np.log(20), np.log(40000), 60))]
    Ns += [3, 100, 256, 257]  # direct-path vectors beside FMM ones

    def run(env):
        with monkeypatch.context() as m:
            for k, v in env.items():
                m.setenv(k, v)
            p = lib.RaggedPlan(Ns, 64)
        u = make_input(p.total, "gauss", 4)
        pre = make_input(p.total, "uniform", 5)
        outs = []
        for d in (0, 1):
            out = pre.copy()
            p(u, out, d)
            outs.append(out)
        return p, outs

    _, want = run({"L2C_OVERLAP": "0"})
    for env in ({}, {"L2C_CHAIN_PRIO": "0"}, {"L2C_OVERLAP": "1", "L2C_CHAIN_PRIO": "1"}):
        _, got = run(env)
        for d in (0, 1):
            assert np.array_equal(got[d], want[d]), (env, d)
    p, _ = run({})
    for d in (0, 1):
        assert p.tuned_config(d)[0] == "default"
        ms = p.autotune(d)
        src, text, mt, md = p.tuned_config(d)
        assert src == "tuned" and mt == ms and 0 < mt <= md and text.startswith("overlap="), text
    u = make_input(p.total, "gauss", 4)
    pre = make_input(p.total, "uniform", 5)
    for d in (0, 1):
        out = pre.copy()
        p(u, out, d)
        assert np.array_equal(out, want[d]), d
