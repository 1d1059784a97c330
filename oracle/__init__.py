"""CPU oracle for the periodic GPW SCF hot path of hqc (ZihangL/hqc v0.1.12).

TEST INFRASTRUCTURE ONLY.  Nothing in the ``hqc_gb300`` product imports this
package; only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg
of ``bench.py`` use it, and only as the checker.

It is a NumPy float64 restatement of the reference algorithm, written in the
streamed (real-space) form: AO values on the grid, rho(r) = sum_pq D_pq
phi_p phi_q, FFT Poisson for Hartree, occupied-pair-density FFT exchange plus
the reference's G=0 Madelung term, LDA and PBE xc, the reference's DIIS /
fixed point SCF with its smearing and chemical-potential search quirks, at
the Gamma point and at a single k-point (complex Bloch AOs, unconjugated
complex DIIS), and the Ewald sums of ``hqc/pbc/potential.py``.  On the odd
grids the reference supports, this form is identical by Parseval to the
reference's rhoG/ERI formulation (``hqc/pbc/solver.py:391-479``).

Parity pin: ``tests/golden/*.npz`` hold outputs of the reference's own
unmodified source, executed by ``tests/golden/make_golden.py`` over a NumPy
stand-in for the JAX API subset it uses.  ``tests/test_oracle_golden.py``
checks this oracle against those vectors.  Analytic forces, which the
reference lacks, are pinned to central finite differences of the
reference's own energies (``pes_gamma`` and ``pes_kpt``, differenced by
``make_golden.py``) and of the oracle's own energy.  GGA-PBE, also absent
from the reference, is checked against the constraints it was built to
satisfy (``tests/test_oracle_xc.py``): "parity unpinned".
"""
