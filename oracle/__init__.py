"""FP64 CPU oracle for the D2IC global finite-element DIC hot path.

TEST INFRASTRUCTURE ONLY.  Nothing in the product package (``d2ic_gb300``)
imports, links or executes anything from this directory.  The only callers
are ``tests/``, ``__graft_entry__.smoke()`` (as a checker) and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py``.

Every function restates, in NumPy float64, the algorithm of the reference
(EmileRouxSMB/D2IC, pure Python on JAX) at the file:line cited in its
docstring.  The reference cannot run in this container (no jax, jaxlib,
im_jax or dm_pix), so the oracle is pinned by

* the reference's own known-answer tests, restated in
  ``tests/test_oracle_pins.py`` (unit-quad pixel->element map
  ``tests/test_pixel_assets.py:6-36``, ZNCC integer shift
  ``tests/test_solver_translation_zncc.py:8-33``, Green-Lagrange stretch
  ``tests/test_strain_smoke.py:10-40``, island removal
  ``tests/test_mask2mesh_smoke.py:8-25``) and the mesh sizes the reference's
  grid mesher gives on the benchmark masks;
* an independent implementation for the one third-party piece of arithmetic:
  the cubic sampler (``im_jax.flat_nd_cubic_interpolate``, un-vendored and
  unpinned) is defined here as the interpolating cubic B-spline with
  'nearest' (edge-replicating) boundary and is checked against
  ``scipy.ndimage.map_coordinates(order=3, mode='nearest')``;
* central finite differences for the analytic gradient that replaces
  ``jax.value_and_grad``.

Whether ``im_jax`` uses exactly this cubic kernel cannot be checked here:
cubic parity with the original reference is UNPINNED (see cubic.py).
"""
