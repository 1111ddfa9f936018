"""The autotuner's two-stage search (geomjax_gb300/autotune.py) with scripted
timings, no GPU: the first stage over tile policies x chains per warp at the
first K-slice value, the second over the other K-slice values with the first
stage's best settings, and the fastest of all left in force."""
from geomjax_gb300.autotune import _candidates, _search


def _run(times, ksplits=(0, 1, 2, 4)):
    cands = _candidates(((0, -1), (64, -1)), (0, 2), ksplits[0])
    state = {"current": None, "applied": []}

    def apply(c):
        state["current"] = c
        state["applied"].append(c)

    def measure():
        c = state["current"]
        return times(c["gemm_tiling"], c["chol_chains_per_warp"], c["gemm_ksplit"])

    return _search(cands, ksplits, apply, measure), state


def test_second_stage_uses_the_first_stages_best():
    def times(tiling, cpw, ks):
        base = {((64, -1), 2): 5.0}.get((tiling, cpw), 9.0)
        return base - {0: 0.0, 1: 0.5, 2: 1.0, 4: 0.2}[ks]

    res, state = _run(times)
    assert len(res.table) == 4 + 3
    assert [c["gemm_ksplit"] for c, _ in res.table[4:]] == [1, 2, 4]
    assert all(c["gemm_tiling"] == (64, -1) and c["chol_chains_per_warp"] == 2
               for c, _ in res.table[4:])
    assert res.best == {"gemm_tiling": (64, -1), "chol_chains_per_warp": 2, "gemm_ksplit": 2}
    assert res.ms_per_transition == 4.0
    assert state["current"] == res.best  # the winner is left in force


def test_first_stage_winner_kept_when_no_split_is_faster():
    res, _ = _run(lambda tiling, cpw, ks: 3.0 if (tiling, cpw, ks) == ((0, -1), 0, 0) else 4.0)
    assert res.best == {"gemm_tiling": (0, -1), "chol_chains_per_warp": 0, "gemm_ksplit": 0}


def test_single_k_value_skips_the_second_stage():
    res, _ = _run(lambda tiling, cpw, ks: 1.0, ksplits=(0,))
    assert len(res.table) == 4
