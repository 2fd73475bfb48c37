"""chorus_mhd -- GB300 (sm_103a) FP64 implementation of CHORUS-MHD's
residual-and-time-step hot path, behind a C-ABI (include/chorus_gpu.h).

Host-side mirror of the reference interface: ``Mesh`` (setup chain), ``Solver``
(compresid / RK_S5P3 / FiveStageRk / correct_B_via_curl_Az / iterations), the
synthetic-case writer ``meshgen``.
"""
from . import meshgen  # noqa: F401
from ._lib import ChorusError, load  # noqa: F401
from .solver import Mesh, Plot, Solver, plot_filename, reference_layout_sizes  # noqa: F401
from .batch import Batch  # noqa: F401
from . import serve  # noqa: F401
