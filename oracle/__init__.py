"""CPU oracle for the DQMC sweep hot path -- TEST INFRASTRUCTURE ONLY.

Nothing in the product (``latticeqmc_gb300``) imports this package.  It is used only by
``tests/``, by ``__graft_entry__.smoke()`` and by the CPU-baseline leg of ``bench.py``, as
the checker the CUDA engine is compared against -- never as the thing measured or shipped.

Modules
-------
compat   numpy restatement of the reference's fast sweep ``LatticeQMC._update_step``
         (lqmc/lqmc.py:156-185, :301-347), defects included.  Pinned: bit-identical to
         the reference's recorded decisions, ratios and G (tests/golden/compat_*.npz).
dqmc     project-written textbook FP64 DQMC (ratio/update/wrap with the correct
         conventions, pre-pivoted QR/UDV stabilisation, Wick measurements).  Pinned
         against the reference's determinant-mode ratios (tests/golden/det_*.npz), the
         U=0 known answer (lqmc/tools.py:193-200) and the exact diagonalisation in ``ed``.
ed       Trotterised Fock-space exact diagonalisation of small Hubbard clusters.
philox   Philox4x64-10 counter-based generator, pinned against numpy's ``Philox``.
"""
