"""CPU oracle for the block-DDA solve path -- TEST INFRASTRUCTURE ONLY.

Nothing in the product imports this package.  Only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py`` (its ``cpu_baseline`` leg and the
``--impl reference`` arm) use it, and there only to check results or as the timed
CPU restatement of the reference algorithm, never as the thing measured on the
GPU.

Contents (each function cites the reference file:line it restates; paths are
relative to the nmoteki/block-DDA source tree):

* ``mbt``      -- the Green tensor block (``mvp_fft/application_function.cpp``),
                  the literal 1-D multilevel block-Toeplitz (MBT) projection
                  (``BT_fft``/``BT_pad``/``BT_reconstruct``/``MBT_fft_init``/
                  ``MBT_fft_mvp``), dense assembly, and the 2x-padded 3-D FFT
                  restatement of the same operator.
* ``krylov``   -- ``qr_reduced`` and the six block solvers
                  (COCG-RQ, BiCGSTAB, BiCGGR, each with and without Jacobi).
* ``physics``  -- target file reader, incident fields, DIAG_A, cross sections.
* ``rng``      -- libstdc++ ``default_random_engine`` + ``uniform_real_distribution``
                  as used by ``Incident_Wave::set_random_incident_directions``.

Parity pins: the f=1 integer known-answer table of
``module_tests/mvp_fft_tests/mvp_fft_example.cpp:37-103`` pins the BT_fft
ordering; the recorded run ``result.dat:14-38`` (f=3 block COCG-RQ-Jacobi on
``DDA_target_0_agg_N512``) pins the solver + cross-section chain end to end;
``result.dat:42`` (MAC_mie) and the reference's own ``gmie`` built under
``oracle/_ref`` pin the polarizability.  See ``tests/golden/make_golden.py``.
"""
