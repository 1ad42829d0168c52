"""GB300-native NUTS sampler with CmdStan's sampling interface.

The compute path is the CUDA library ``_lib/libgnuts.so`` (include/gnuts.h);
``gnuts`` is its Python mirror.
"""
from .gnuts import (Model, Fit, GnutsError, default_args, load, SAMPLER_COLUMNS, METRICS,  # noqa: F401
                    PRECISION_FP64, PRECISION_MIXED)
