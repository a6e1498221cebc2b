"""GB300-native kernel low-rank pipeline: bandwidth calibration, block randomly
pivoted Cholesky and bistochastic EVD on one GPU, behind the C ABI of
include/kevd.h (libkevd.so, built by ``python -m kernel_evd_gb300.build``); the
reference's HDF5 stage files through include/kevd_h5.h (libkevdh5.so, ``h5``)."""
from . import _lib  # noqa: F401
from ._lib import KEVD_FP64, KEVD_MIXED, KevdError  # noqa: F401

__all__ = ["api", "h5", "KevdError", "KEVD_FP64", "KEVD_MIXED"]
