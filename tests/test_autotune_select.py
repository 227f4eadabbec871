"""The autotuner's selection rules (CPU): fastest candidate that reaches the
tolerance; smallest residual for omega; parameter copies."""
from flowlab_gb300 import autotune, configs, native


def test_fastest_converged_candidate_wins():
    res = [({"mg_coarsest": 4}, {"ms": 1.0, "rel_max": 2e-6, "cycles": 5}),
           ({"mg_coarsest": 8}, {"ms": 1.2, "rel_max": 9e-7, "cycles": 4}),
           ({"mg_coarsest": 16}, {"ms": 1.1, "rel_max": 8e-7, "cycles": 4}),
           ({"mg_coarsest": 32}, {"ms": 0.9, "rel_max": -1.0, "cycles": 20})]
    best = autotune.pick_multigrid(res, 1e-6)
    assert best[0] == {"mg_coarsest": 16}
    assert autotune.pick_multigrid(res[:1], 1e-6) is None


def test_omega_by_residual():
    assert autotune.pick_omega([(1.7, 1e-3), (1.9, 2e-4), (1.95, 2e-4)]) == 1.9


def test_with_params_copies():
    base = configs.plume_params()
    p = autotune.with_params(base, mg_coarsest=16)
    assert p.mg_coarsest == 16 and base.mg_coarsest == 8 and p.tol == base.tol
    assert autotune.cache_key(p, 256, 128) == "mg:256x128:mixed"
    assert autotune.cache_key(configs.karman_params(), 128, 128) == "rb:128x128:f32"


def test_tail_side_chosen_by_time_after_the_constants(monkeypatch):
    """tune_multigrid: the fastest converged (mg_coarsest, mg_coarse_sweeps),
    then the tail's first level by time alone, with those constants."""
    seen = []

    def fake_measure(scene, prm, steps, warmup, device):
        seen.append((prm.mg_coarsest, prm.mg_coarse_sweeps, prm.mg_tail_side))
        ms = 1.0 + 0.01 * prm.mg_coarsest + 0.001 * prm.mg_coarse_sweeps
        if prm.mg_tail_side:
            ms = {16: 0.95, 32: 0.90, 64: 0.97}[prm.mg_tail_side]
        return {"ms": ms, "rel_max": 5e-7, "cycles": 4}

    monkeypatch.setattr(autotune, "measure_steps", fake_measure)
    best, results = autotune.tune_multigrid(None, configs.plume_params(tol=1e-6))
    assert best == {"mg_coarsest": 4, "mg_coarse_sweeps": 8, "mg_tail_side": 32}
    assert len(results) == 12
    assert seen[-3:] == [(4, 8, 16), (4, 8, 32), (4, 8, 64)]


def test_warm_start_gate():
    """The learned warm start stays attached only when it makes the step
    faster and still reaches the tolerance."""
    plain = {"ms": 0.58, "cycles": 4.2, "rel_max": 9e-7, "rel0_mean": 6e-3}
    slow = {"ms": 1.33, "cycles": 4.2, "rel_max": 9e-7, "rel0_mean": 4e-3}
    fast = {"ms": 0.50, "cycles": 3.0, "rel_max": 9e-7, "rel0_mean": 4e-4}
    missed = {"ms": 0.40, "cycles": 3.0, "rel_max": 2e-6, "rel0_mean": 4e-4}
    assert autotune.warm_start_pays(plain, slow, 1e-6)[0] is False
    assert autotune.warm_start_pays(plain, fast, 1e-6)[0] is True
    assert autotune.warm_start_pays(plain, missed, 1e-6)[0] is False
