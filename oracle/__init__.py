"""CPU oracle for the multilayer quasi-geostrophic time step (test infrastructure).

This package is the checker, not the product: only ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py`` may import it.  It restates, in NumPy/SciPy
(float64 by default, any float dtype on request), the arithmetic of somax's QG hot path:

* ``somax/_src/models/qg/baroclinic.py:135-195``   (modal PV inversion, RHS, BCs)
* ``somax/_src/models/qg/barotropic.py:113-157``   (Poisson inversion, RHS, BCs)
* ``somax/_src/core/transforms.py:172-224``        (layer <-> mode matrices)
* ``somax/_src/core/model.py:39-88``               (BC on every stage input, RK stepping)
* ``somax/_src/models/qg/baroclinic.py:197-228``   (diagnostics)
* ``tests/models/test_qg_baroclinic.py:293-312``   (gradients: ``adjoint.py`` gives the float64
  derivatives that JAX autodiff gives the reference, from exact or central differences)

The operators themselves live in finitevolx v0.0.39 / spectraldiffx v0.0.10, which are not
vendored in the reference; they are restated here from the published methods (Arakawa 1966,
DST-I Helmholtz, 5-point Laplacian) and pinned against the printed outputs of the
reference's tutorials (see ``tests/golden``).
"""

from . import adjoint, qg  # noqa: F401
