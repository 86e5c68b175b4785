"""GB300-native (sm_103a) XPCS g2 correlator with the dynamix correlator API.

``from dynamix_gb300.correlator import MatMulCorrelator`` is a drop-in for
``dynamix.correlator.dense.MatMulCorrelator``; the arithmetic runs in the CUDA
kernels of ``libdynamix_g2.so`` (C ABI: ``include/dynamix_g2.h``).
"""
__version__ = "0.1.0"
