"""Maps engine parameters onto the oracle's, for whole-step comparisons."""
from oracle import params_from_engine as oracle_params  # noqa: F401
