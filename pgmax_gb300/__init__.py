"""pgmax_gb300: a GB300-native loopy belief propagation engine behind PGMax's BP interface.

Modules mirror PGMax's: `vgroup`, `factor`, `fgroup`, `fgraph`, `infer`. Graph construction is host
NumPy; every belief-propagation computation runs in libpgbp's sm_103a kernels through the C ABI of
include/pgbp.h (`native`, `engine`).
"""

from . import factor, fgraph, fgroup, infer, utils, vgroup

__version__ = "0.1.0"
