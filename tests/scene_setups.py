"""Maps engine parameters onto the oracle's, for whole-step comparisons."""
from flowlab_gb300 import native
from oracle import SOLVER_MG, SOLVER_RBSOR


def oracle_params(p):
    return dict(cflTarget=p.cfl_target, dtMax=p.dt_max, rho=p.rho, macCormack=int(p.scheme == native.FL_MACCORMACK),
                solver=SOLVER_MG if p.solver == native.FL_SOLVER_MG else SOLVER_RBSOR,
                pressureIters=p.pressure_iters, mgMaxCycles=p.mg_max_cycles, omega=p.omega, tol=p.tol,
                dyeDecay=tuple(p.dye_decay), beta=p.beta, alpha=p.alpha, confinement=p.confinement,
                mgPre=p.mg_pre, mgPost=p.mg_post, mgCoarseSweeps=p.mg_coarse_sweeps, mgCoarsest=p.mg_coarsest,
                mgOmega=p.mg_omega)
