"""The autotuner's search and cache logic, driven by a stand-in batch whose
solve times come from a table (no GPU)."""
import pytest

from minife_gb300 import autotune


class _Res:
    def __init__(self, t, status=0, op="padded"):
        self.times = (0.0, 0.0, 0.0, 0.0, t)
        self.status = status
        self.inner_operator = op


class FakeBatch:
    """solve() time: a function of the current shape/chunk (capped runs) or
    of refine_k (full runs)."""

    def __init__(self):
        self.dims = [(4, 5, 6), (7, 3, 9)]
        self.tuning = None
        self.calls = []

    def set_tuning(self, rows, stages, chunk):
        self.tuning = (rows, stages, chunk)

    def solve(self, max_iter, tol, tol_mode, precision, refine_k):
        rows, stages, chunk = self.tuning
        self.calls.append((self.tuning, max_iter, tol, refine_k))
        if tol == 0.0:  # capped probe: shape (128, 3) and chunk 16384 are fastest
            t = 1.0 + 0.1 * abs(rows - 128) / 128 + 0.05 * abs(stages - 3) + \
                0.01 * abs(chunk - 16384) / 16384
            return None, [_Res(t, 5)] * 2
        # full solves: refine_k 100 and 200 fastest but do not converge, 50 next
        t = {25: 3.0, 50: 2.0, 100: 1.0, 200: 0.5}[refine_k]
        return None, [_Res(t, 0 if refine_k < 100 else 5)] * 2


@pytest.fixture
def cache(tmp_path, monkeypatch):
    monkeypatch.setenv("MFE_TUNE_CACHE", str(tmp_path / "tune.json"))
    monkeypatch.setattr(autotune, "_device_key", lambda: "fake/sm1")
    return tmp_path / "tune.json"


def test_search_picks_fastest_converging(cache):
    b = FakeBatch()
    cfg = autotune.tune_batch(b, probe_iters=5, reps=1)
    assert (cfg["spmv_rows"], cfg["spmv_stages"], cfg["chunk_rows"]) == (128, 3, 16384)
    assert cfg["refine_k"] == 50           # 100 and 200 are faster but did not converge
    assert b.tuning == (128, 3, 16384)     # applied to the batch
    assert not cfg["cached"] and cache.exists()
    assert all(c[1] == 5 for c in b.calls if c[2] == 0.0)  # capped probes


def test_cache_hit_skips_search(cache):
    b = FakeBatch()
    autotune.tune_batch(b, probe_iters=5, reps=1)
    b2 = FakeBatch()
    cfg = autotune.tune_batch(b2, probe_iters=5, reps=1)
    assert cfg["cached"] and b2.calls == [] and b2.tuning == (128, 3, 16384)
    assert autotune.lookup(b.dims, "mixed")["refine_k"] == 50
    # another workload or precision is another entry
    assert autotune.lookup([(4, 5, 6)], "mixed") is None
    assert autotune.lookup(b.dims, "f64") is None


def test_signature_ignores_box_order(cache):
    assert autotune.signature([(1, 2, 3), (4, 5, 6)], "mixed") == \
        autotune.signature([(4, 5, 6), (1, 2, 3)], "mixed")


class StencilBatch(FakeBatch):
    """Every box passes the stencil check: the SpMV shape has no effect."""

    def solve(self, max_iter, tol, tol_mode, precision, refine_k):
        t, res = super().solve(max_iter, tol, tol_mode, precision, refine_k)
        return t, [_Res(r.times[4], r.status, "stencil") for r in res]


def test_stencil_batch_skips_shape_search(cache):
    b = StencilBatch()
    cfg = autotune.tune_batch(b, probe_iters=5, reps=1)
    shapes = {c[0][:2] for c in b.calls if c[2] == 0.0}
    assert shapes == {autotune.SHAPES[0]}   # one capped trial, then chunks only
    assert cfg["inner_operator"] == "stencil" and cfg["refine_k"] == 50


class _Vec:
    """Stand-in for a device vector: shape, new_zeros and zero_."""

    shape = (8, 32)

    def new_zeros(self, shape):
        return _Vec()

    def zero_(self):
        return self


class _Box:
    box = (16, 16, 16)


class _CG:
    def __init__(self, t, status):
        self.total_time = t
        self.status = status
        self.times = (0.0, 0.0, 0.0, 0.0, t)


def test_tune_mixed_searches_refine_k_10_to_50(cache, monkeypatch):
    """refine_k over 10..50 x inner_tol: the fastest converging pair wins,
    is cached, and a second call is a cache hit with no solves."""
    import minife_gb300 as M
    seen = []

    def fake_cg(A, b, x, max_iter, tol, tol_mode, precision, refine_k, inner_tol):
        seen.append((refine_k, inner_tol))
        t = 1.0 + abs(refine_k - 30) / 100 + (0.05 if inner_tol == 0.1 else 0.0)
        return _CG(t, 5 if refine_k == 10 else 0)  # k = 10 fails to converge

    monkeypatch.setattr(M, "cg_solve", fake_cg)
    cfg = autotune.tune_mixed(_Box(), _Vec(), reps=1)
    assert (cfg["refine_k"], cfg["inner_tol"]) == (30, 0.01) and not cfg["cached"]
    assert {k for k, _ in seen} == set(autotune.SINGLE_REFINE_K)
    assert min(autotune.SINGLE_REFINE_K) == 10 and max(autotune.SINGLE_REFINE_K) == 50
    seen.clear()
    cfg2 = autotune.tune_mixed(_Box(), _Vec(), reps=1)
    assert cfg2["cached"] and seen == [] and cfg2["refine_k"] == 30


def test_tune_multi_picks_z_chunk_then_refine(cache, monkeypatch):
    import minife_gb300 as M
    state = {"zc": 0}
    applied = []

    def fake_set(z):
        state["zc"] = z
        applied.append(z)

    def fake_multi(A, B, X, max_iter, tol, tol_mode, precision, refine_k, inner_tol):
        if tol == 0.0:  # capped probe: z chunk 64 fastest
            t = {8: 1.4, 16: 1.3, 32: 1.1, 64: 1.0}[state["zc"]]
            return [_CG(t, 5)] * 2
        t = {25: 2.0, 50: 1.5, 100: 1.2}[refine_k] + (0.1 if inner_tol == 0.01 else 0.0)
        return [_CG(t, 0)] * 2

    monkeypatch.setattr(M, "set_multi_tuning", fake_set)
    monkeypatch.setattr(M, "cg_solve_multi", fake_multi)
    cfg = autotune.tune_multi(_Box(), _Vec(), _Vec(), reps=1)
    assert (cfg["z_chunk"], cfg["refine_k"], cfg["inner_tol"]) == (64, 100, 0.1)
    assert applied[-1] == 64
    applied.clear()
    cfg2 = autotune.tune_multi(_Box(), _Vec(), _Vec(), reps=1)
    assert cfg2["cached"] and applied == [64]
