"""CPU oracle for the backward-Euler stable neo-Hookean FEM path of simkit.

TEST INFRASTRUCTURE ONLY.  This package is an FP64 numpy/scipy restatement of
the reference algorithm, used as the checker for the CUDA path.  Only the test
suite, ``__graft_entry__.smoke()`` and the CPU-baseline legs of ``bench.py``
may import it.  The product package ``simkit_gb300`` never imports, links or
executes anything in here.

Parity is pinned: ``tests/golden/make_golden.py`` imports the reference itself
and writes fixtures under ``tests/golden/``; ``tests/test_oracle_pin.py``
checks every function here against those fixtures.

Modules
-------
snh       element tier (energy density, PK1, 9x9 F-Hessian) and the x tier
psd       batched eigen-floor PSD projection
fem       deformation Jacobian, volumes, lumped mass, gravity, Lame conversion
solvers   Armijo backtracking, Newton (sparse direct solve), backward Euler
rollout   free-DOF-eliminated backward-Euler rollout with a relative-residual stop
"""

from . import snh, psd, fem, solvers, rollout  # noqa: F401
