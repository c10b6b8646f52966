"""GB300 (sm_103a) SuBSENSE, PAWCS, LOBSTER, ViBe and PBAS background subtraction with LITIV's interface.

The compute path is the in-tree CUDA library ``_build/liblvbgs.so`` (C-ABI in include/lvbgs.h);
this package is its host-side mirror of the reference's BackgroundSubtractorSuBSENSE,
BackgroundSubtractorPAWCS, BackgroundSubtractorLOBSTER, BackgroundSubtractorViBe and BackgroundSubtractorPBAS
interfaces.
"""
from .bgs import (BackgroundSubtractorLOBSTER, BackgroundSubtractorPAWCS, BackgroundSubtractorPBAS,  # noqa: F401
                  BackgroundSubtractorSuBSENSE, BackgroundSubtractorViBe, LvException, batch_apply, lbsp_compute2)
from .precache import DataPrecacher, DevicePacket  # noqa: F401
from .synth import SyntheticStream  # noqa: F401
from . import _lib  # noqa: F401
