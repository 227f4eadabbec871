"""How good a pressure warm start must be to save a V-cycle on the 1024^2
plume at 1e-6 (the benchmark's solve), measured on the float32 oracle: no
GPU. The plume is stepped 12 times from its reset; the 13th step's solve
(double-float defect correction, V(3,3), 16 coarse sweep pairs, 8x8
coarsest level) is then started from candidate guesses and the relative
residual recorded after each V-cycle (one-cycle solves chained: each
restarts from the pressure the last one left, which is the same
computation as one longer solve).

The result bounds any learned warm start: a V(3,3) cycle contracts the
residual ~20x, so a guess saves a cycle only when it is better than ~90%
of the exact per-step correction; neither the second-order extrapolation
nor the exact correction on a 2x coarser grid reaches that. Run with -s
to see the table."""
import numpy as np
import pytest
from scipy.ndimage import zoom

from flowlab_gb300 import configs
from oracle import Oracle, params_from_engine as oracle_params

N = 1024
TOL = 1e-6


def coarse(d, f):
    """The correction seen at a grid f times coarser: block means, then
    bilinear back to the fine grid."""
    a = d.reshape(N, N).reshape(N // f, f, N // f, f).mean(axis=(1, 3))
    return zoom(a, f, order=1).ravel()


@pytest.mark.slow
def test_warm_start_needed_to_save_a_cycle():
    g, f, patch = configs.plume(N)
    prm = configs.plume_params()
    o = Oracle("f32")
    sim = o.simulation(N, N, 1, **oracle_params(prm))
    sim.set_fields(f.u, f.v, f.p, f.label, f.dye)
    sim.set_patch(patch.i0, patch.j0, patch.nx, patch.ny, patch.data)
    hist = []
    for _ in range(14):
        sim.step()
        hist.append(sim.get_p64().copy())
    div, scale = sim.get_div(), float(np.float32(sim.scale()))
    pc, pp, pp2 = hist[-1], hist[-2], hist[-3]
    fl = f.label == 0
    delta = pc - pp
    extrap = np.where(fl, 2 * pp - pp2, pp)

    def history(w, most=6):
        out, p = [], w
        for _ in range(most):
            p, _, rr = o.mg_solve_df(N, N, p, div, f.label, scale, 1, TOL, pre=3, post=3, coarse=16, coarsest=8)
            out.append(rr)
            if rr <= TOL:
                break
        return out

    cands = {
        "previous pressure": pp,
        "2p(n) - p(n-1)": extrap,
        "exact x 0.5": pp + 0.5 * delta,
        "exact x 0.9": pp + 0.9 * delta,
        "exact at 512^2": pp + np.where(fl, coarse(delta, 2), 0),
        "exact at 256^2": pp + np.where(fl, coarse(delta, 4), 0),
        "extrapolation + exact at 256^2": extrap + np.where(fl, coarse(pc - extrap, 4), 0),
    }
    cycles = {}
    for name, w in cands.items():
        h = history(w)
        err = np.linalg.norm((w - pc)[fl]) / np.linalg.norm(delta[fl])
        cycles[name] = len(h)
        print("%-32s error %.3f  cycles %d  residuals %s" % (name, err, len(h), " ".join("%.2e" % r for r in h)))
        assert h[-1] <= TOL
    base = cycles["previous pressure"]
    # nothing short of ~90% of the exact correction saves a cycle
    for name in ("2p(n) - p(n-1)", "exact x 0.5", "exact x 0.9", "exact at 512^2", "exact at 256^2",
                 "extrapolation + exact at 256^2"):
        assert cycles[name] == base, (name, cycles)
