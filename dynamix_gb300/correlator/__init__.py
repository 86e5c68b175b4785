"""Correlator API, mirroring ``dynamix.correlator`` (dense, event, sparse)."""
from .common import BaseCorrelator  # noqa: F401
from .dense import (CorrelationResult, CublasMatMulCorrelator, DenseCorrelator,  # noqa: F401
                    MatMulCorrelator, py_dense_correlator)
from .event import EventCorrelator, FramesCompressor  # noqa: F401
from .intensity import SparseCorrelator  # noqa: F401
