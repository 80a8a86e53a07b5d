"""CPU FP64 oracle for the DG-FEM RHS operators (TEST INFRASTRUCTURE ONLY).

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py`` (its CPU
baseline and ``--impl reference`` legs) may import this package, and only as
the checker or the timed CPU baseline; the product package
``actx_dgfem_suite_gb300`` never imports it.

What it restates (reference files, paths inside kaushikcfd/actx_dgfem_suite):

* ``oracle.rhs.wave_rhs`` -- ``actx_dgfem_suite/equations/wave.py:80-200``
  (``wave_flux`` and ``wave_operator``), evaluated unfused exactly as written:
  ``inverse_mass(-c weak_div(v), -c weak_grad(u)) + inverse_mass(face_mass(flux))``.
* ``oracle.rhs.euler_rhs`` -- grudge's ``EulerOperator.operator`` with
  ``flux_type="lf"`` and ``InviscidWallBC`` as configured at
  ``actx_dgfem_suite/equations/euler.py:168-179``.
* ``oracle.rhs.maxwell_rhs`` -- grudge's ``MaxwellOperator.operator`` with
  epsilon = mu = 1, ``flux_type=0.5`` and PEC on all boundaries as configured at
  ``actx_dgfem_suite/equations/maxwell.py:55-70``.

grudge, meshmode and modepy are un-vendored, unpinned git dependencies of the
reference (``.test-conda-env.yml:17-25``) and are absent here; their
algorithms are restated from their published definitions (nodal DG on
simplices, Hesthaven & Warburton 2008).

Independence from the product: no module here imports the product package.
The reference element is the oracle's own (``oracle.refelem``): GLL points
from NumPy's Legendre roots, the recursive node family placed from its
definition (vertices, GLL edge points, centroids, and the order-4
face-interior nodes in closed form), products of Legendre polynomials as
the modal basis and collapsed Gauss-Legendre quadrature, all in 32-digit
arithmetic (mpmath); the matrices are assembled by quadrature in the same
precision (``oracle.refops``); exterior face values are found by matching physical node
coordinates (``oracle.geometry``), not through the product's gather index.
Only the mesh (vertex coordinates and element vertex lists) and the state
arrays are inputs shared with the product; the tests check that the product's
nodes sit at the oracle's node coordinates, in the same order.

Parity status: the reference ships no golden vectors, known-answer tests or
fixtures for this path (``test/test_dgfem_opt_freeze.py:1-4`` is a
placeholder) and cannot run here, so parity with the reference's own numbers
is UNPINNED.  The oracle is pinned instead by known-answer tests
(polynomial exactness, free-stream preservation, discrete conservation,
convergence to the analytic cavity mode) in ``tests/test_oracle_kat.py``,
and its wave operator by the reference's own ``wave_operator`` code, run
on stand-in modules over this package's primitives
(``tests/golden/make_reference_equations.py``): same result to the bit.
"""
