"""CPU oracle for the propagation hot path - TEST INFRASTRUCTURE ONLY.

A complex128 numpy/scipy restatement of the reference's algorithms (each function cites
the reference file:line it follows). It checks the GPU path; it is never the thing
measured or shipped. Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg
of ``bench.py`` may import it.

Parity anchors (the reference ships no golden vectors for this path):
  * analytic hydrogen eigenvalues E_n = -1/(2 n^2) for the assembled operator;
  * the pIRAM fixture ``core/krylov/piram/piram/qdotmatrix.dat`` + ``init.dat`` (reduced to
    ``tests/golden/qdot_piram.npz`` by ``tests/golden/make_golden.py``), whose lowest
    eigenvalues the oracle pIRAM must reproduce;
  * pAMP's 2x2 Pade test (``core/krylov/pamp/pampwrapper.h:79-101``) and the exact
    ``scipy.linalg.expm`` of the dense operator;
  * an independent B-spline evaluation (``scipy.interpolate.BSpline``) for the radial
    matrix elements.
"""
