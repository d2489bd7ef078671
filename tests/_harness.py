"""Test access to the oracle (oracle/pyoracle.py): the checker, never the product."""
import sys
from pathlib import Path

_ORACLE = Path(__file__).resolve().parents[1] / "oracle"
if str(_ORACLE) not in sys.path:
    sys.path.insert(0, str(_ORACLE))

from pyoracle import *  # noqa: E402,F401,F403
from pyoracle import (ORACLE_DIR, ORACLE_LIB, REF_LIB, REF_SRC, OracleSim, build_oracle, consts_of, oracle,  # noqa: E402,F401
                      ref, ref_available, sim_arrays)
