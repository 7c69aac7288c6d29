"""CPU oracle for the SU(2) block-DMRG superblock step.

TEST INFRASTRUCTURE ONLY.  This package restates, in numpy, the algorithm of the
reference Fortran code (cfengno1/Hofstadter_Hubbard_TSC, ``code/*.f90``) for the
hot path: the superblock matvec ``model_wave`` and its term kernels
(``code/mat_vec.f90``), ``hmerge``, the Lanczos solver ``lanczos_memo_new``
(``code/lanczos.f90``), the reduced density matrix and per-sector truncation
(``code/get_den.f90``), operator renormalisation ``update_trun_dia/ndia`` and the
block enlargement of ``code/update.f90`` / ``code/get_ham.f90``, and the
wavefunction transformation ``wave_trans_LR/RL`` (``code/warm_up.f90``).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import it, and only as the checker.  The product path
(``hofstadter_hubbard_tsc_gb300``) never imports it.

Parity status: the reference ships no tests, golden vectors or published
energies for this path and no Fortran compiler is available, so the oracle is
"parity unpinned" against the reference itself.  It is pinned instead by
physics known-answer tests: exact diagonalisation of small flux ladders, the
U=0 free-fermion energy, 6j identities and Hermiticity of the matvec
(``tests/test_oracle_*.py``).
"""
