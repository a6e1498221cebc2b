"""CPU oracle for the kernel low-rank pipeline (FP64 NumPy restatement).

This package is TEST INFRASTRUCTURE.  Only ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline legs of ``bench.py`` may import it, and only as the
reference the GPU results are compared with (or as the timed CPU baseline); the
product path in ``kernel_evd_gb300`` never imports, links or executes anything
here.

Modules and the reference code they restate:

* ``ks``        -- KS ETDRK4 generator (ks_datagen.py:21-101)
* ``kernel``    -- Hankel / dense sample views and kernel blocks (ks_arpclm.cu:242-280)
* ``calibrate`` -- pair-sum sweep and bandwidth selection (ks_bandwidth.cu:181-325, :612-656)
* ``rpchol``    -- block RPCholesky, stored factor (ks_arpclm.cu:197-564)
* ``evd``       -- bistochastic normalisation + EVD (ks_kevd.cu, README_kevd.md:20-69)
* ``dense``     -- dense FP64 EVD (ks_reference.py:24-58)
* ``philox``    -- counter-based uniforms shared with the device sampler

Pinning: ``ks``, ``kernel`` (Hankel order) and ``dense`` are checked against
outputs of the reference's own Python programs run on small inputs
(``tests/golden``).  The calibration, RPCholesky and factor-EVD restatements
have no reference-produced vectors (the reference ships no tests and its CUDA
programs cannot be built here); they are pinned indirectly: a full-rank
factorisation must reproduce the reference's dense EVD.
"""
