"""CPU oracle for the g2 correlator -- TEST INFRASTRUCTURE ONLY.

This package restates, on the CPU, the arithmetic of the dynamix correlators
(``dynamix/correlator/dense.py``, ``event.py``, ``intensity.py`` and the OpenCL
kernels under ``dynamix/resources/opencl/``) so that the GPU product can be
checked against it.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may import it, and
only as the checker or the timed CPU baseline.  The product package
(``dynamix_gb300``) never imports anything from here and has no CPU fallback.

Pinning: ``g2_oracle.matmul_correlator_port`` and ``g2_oracle.g2_exact`` are
checked in ``tests/test_oracle.py`` against golden vectors produced by running
the reference's own ``MatMulCorrelator`` and ``FramesCompressor`` (script:
``tests/golden/make_golden.py``).  The OpenCL kernels are also compiled from the
reference's ``.cl`` sources through a small C shim (``oracle/clshim``) and the
restatements of the event, CSR and dense kernels are checked against them.
"""
