"""synchrad_gb300: SynchRad's radiation integral on GB300 (sm_103a).

A drop-in for the reference's Python API (``from synchrad_gb300.calc import
SynchRad``) backed by hand-written CUDA kernels in ``libsynchrad_gb300.so``,
whose C ABI is declared in ``include/synchrad_gb300.h``.
"""
__version__ = "0.1.0"

from .calc import SynchRad  # noqa: E402,F401
from .utils import Utilities, J_in_um, r_e, omega_1m, energy_1m_eV  # noqa: E402,F401
