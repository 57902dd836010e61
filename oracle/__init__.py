"""
CPU oracle for the DFT-D4 dispersion path (TEST INFRASTRUCTURE ONLY).

This package restates tad-dftd4's ``dftd4()`` path in float64 PyTorch on the
CPU.  It is the checker the CUDA path is compared against, and the CPU arm of
the benchmark.  Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``
(its CPU-baseline leg and ``--impl reference``) may import it.  The product
package never does: it has no CPU fallback.

Parity status
-------------
* Pinned: the in-tree maths of tad-dftd4 (reference polarisabilities, charge
  scaling, Gaussian weights for D4 and D4S, C6 integration, BJ two-body
  energy, ATM three-body energy, padding masks, autograd gradients).  The
  fixtures under ``tests/golden`` were produced by running tad-dftd4's own
  modules, and ``tests/test_oracle_golden.py`` checks this oracle against
  them.
* Unpinned: the D4 coordination number and the EEQ charges.  tad-dftd4 takes
  them from ``tad-mctc==0.7.0`` and ``tad-multicharge==0.5.0``, which are not
  in the reference tree.  They are restated here from the published method
  (Caldeweyher et al., J. Chem. Phys. 150, 154122 (2019)), and their element
  tables are placeholders unless real ones are supplied (see
  ``tad-dftd4_gb300/data/make_tables.py``).
"""

from .d4_oracle import *  # noqa: F401,F403
