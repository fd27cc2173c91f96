"""CPU FP64 oracle for the Bloch-Torrey signal path -- TEST INFRASTRUCTURE ONLY.

This package is a numpy/scipy restatement of the reference's solve path
(van-dang/DMRI-FEM-Cloud, ``DmriFemLib.py``).  It exists to check the CUDA
engine, and it is imported only by ``tests/``, ``__graft_entry__.smoke()`` and
the ``cpu_baseline`` / ``--impl reference`` legs of ``bench.py``.  The product
(the ``dmri-fem-cloud_gb300`` package and its ``libbtgpu.so``) never imports,
links or executes anything in here.

Why a restatement: the reference's arithmetic lives in DOLFIN 2019.1.0 / FFC /
PETSc (``assemble``, ``KrylovSolver``, ``PETScLUSolver``), none of which is
vendored in the reference nor installable here, so the reference cannot be
run.  The restatement follows the reference's forms line by line:

* ``forms.py``   -- the two-field real "phase" formulation exactly as the UFL
  forms state it (``DmriFemLib.py:41-50, 58-145, 240-254``) and the equivalent
  complex duplicated-interface-node formulation used by the GPU engine.
* ``loop.py``    -- ``MRI_simulation.solve`` (``DmriFemLib.py:878-915``) with its
  exact time-loop semantics (f(t) implicit, f(t_prev) explicit,
  ``while t < T + k``), ``PostProcessing`` signal (``DmriFemLib.py:917-931``).
* ``sequence.py``-- ``MRI_parameters`` (``DmriFemLib.py:800-858``): f(t), the
  b -> q conversion through int_0^T (int_0^s f)^2.
* ``periodic.py``-- the weak pseudo-periodic boundary term (``DmriFemLib.py:
  58-145, 256-323, 386-451, 596-610``): boundary penalty matrix and mirror map.
* ``mesh.py``    -- DOLFIN ``BoxMesh`` (6 tets per cube around the
  (0,0,0)->(1,1,1) diagonal), used by the reference's ``ConvergenceTest``.

Parity pins (see ``tests/test_oracle_pins.py``):

* ``ConvergenceTest.ipynb:245,261-263,353,366-395,423`` -- BoxMesh [-2.5,2.5]^3
  with 16 cubes per axis (the printed hmin 5.413e-01 = sqrt(3)*5/16 identifies
  the run; the n=5 in the cell source is a later edit), D=2e-3, PGSE
  delta=1000 Delta=10000, dt=10, b=1000, g=(0,0,1), MUMPS LU, loop
  ``while t < T``: normalised signal 8.440078e-01 and q, g, hmin to all printed
  digits (``tests/golden/reference_kats.json``); the 216/750 counts of the
  n=5 box pin the BoxMesh layout.
* b = 0 gives a normalised signal of exactly 1 (``ExplicitImplementation.ipynb:437``).
* q = 0 with uniform T2 gives ((1 - k/(2 T2)) / (1 + k/(2 T2)))^N exactly.
* The literal two-field formulation and the duplicated-node complex
  formulation agree to 1e-13 on the same mesh.
"""

from .mesh import box_mesh, region_from_centroids  # noqa: F401
from .sequence import (  # noqa: F401
    PGSE, CosOGSE, Sequence, reference_schedule, bvalue_to_q,
)
from .forms import (  # noqa: F401
    element_geometry, duplicated_system, two_field_system, interface_facets,
)
from .loop import (  # noqa: F401
    solve_duplicated, solve_two_field, OracleResult,
)
from .periodic import weak_periodic  # noqa: F401
