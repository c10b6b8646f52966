"""GB300 (sm_103a) SuBSENSE and PAWCS background subtraction with LITIV's interface.

The compute path is the in-tree CUDA library ``_build/liblvbgs.so`` (C-ABI in include/lvbgs.h);
this package is its host-side mirror of the reference's BackgroundSubtractorSuBSENSE and
BackgroundSubtractorPAWCS interfaces.
"""
from .bgs import BackgroundSubtractorPAWCS, BackgroundSubtractorSuBSENSE, LvException, batch_apply, lbsp_compute2  # noqa: F401
from .synth import SyntheticStream  # noqa: F401
from . import _lib  # noqa: F401
