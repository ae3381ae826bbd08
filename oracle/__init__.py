"""CPU oracle for the AutoPDEx solve path — TEST INFRASTRUCTURE ONLY.

This package restates, in float64 NumPy/SciPy (with ``torch.func`` for the
element derivatives), the algorithm AutoPDEx runs for its Newton solve path:

* ``mesh``      structured meshes, Gauss-Legendre rules, Lagrange shape functions
                and the boundary selectors (mesher.py, seeder.py, spaces.py,
                geometry.py of AutoPDEx),
* ``elements``  the element routines, derived by automatic differentiation the way
                AutoPDEx derives them (models.py, assembler.py),
* ``newton``    COO assembly with duplicates, the SciPy CSR conversion with
                Dirichlet row/column deletion, ``spsolve``, and the damped Newton
                loop with its stopping rules (solver.py, utility.py),
* ``nn``        the learned preconditioner's U-Net in float64 (forward and
                gradients), the checker of the tensor-core kernels,
* ``corc``      ctypes front end of ``c/orc.c``: the neo-Hooke brick element in
                closed form and a Jacobi-PCG on CSR, in plain C with OpenMP
                (built by ``build_oracle.py``), checked against ``elements`` and
                used as the timed CPU baseline.

Only ``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` leg of
``bench.py`` may import it, and only as the checker.  The GPU backend in
``autopdex_gb300`` never imports or calls anything here.

Parity pin: ``tests/test_oracle_golden.py`` reproduces the golden values of the
reference's own tests (``tests/test_dicts_as_dofs_user_potential.py:63`` and
``tests/test_user_elem_impl_diff_and_adaptive_load_step.py:153``).
"""
