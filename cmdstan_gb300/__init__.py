"""GB300-native NUTS sampler with CmdStan's sampling interface.

The compute path is the CUDA library ``_lib/libgnuts.so`` (include/gnuts.h);
``gnuts`` is its Python mirror.
"""
from .gnuts import (Model, Fit, Flow, GnutsError, default_args, learned_args, train_args, load, summary,  # noqa: F401
                    summary_columns, SAMPLER_COLUMNS, METRICS, PRECISION_FP64, PRECISION_MIXED)
