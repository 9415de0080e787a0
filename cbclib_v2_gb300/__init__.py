"""GB300-native (sm_103a) implementation of cbclib_v2's streak-model rasteriser
``draw_lines`` behind the reference's Python signature, with the ``device`` switching
module of the reference README.  Compute runs only in the CUDA library built from
``csrc/`` (C ABI: include/cbc_draw_lines.h)."""
from . import device, ndimage, streaks
from .ndimage import accumulate_lines, draw_lines
from .streaks import Lines, StackedStreaks, Streaks

__version__ = '0.1.0'
__all__ = ["device", "ndimage", "streaks", "draw_lines", "accumulate_lines", "Lines", "Streaks", "StackedStreaks"]
