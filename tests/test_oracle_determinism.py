"""The oracle's results do not depend on the number of OpenMP threads: its
inner products are summed in fixed chunks, so CG and BiCGStab (whose erratic
residual on the non-normal D amplifies any rounding difference) give
bit-identical iterates on any host."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROG = r"""
import hashlib, sys
import numpy as np
sys.path.insert(0, {root!r})
from oracle import oracle as O
from tests.gpu_util import rand_spinor
n = 8
rng = np.random.default_rng(95 + n)
g = O.geometry(n)
A = rng.uniform(-np.pi, np.pi, g.n_links)
D = O.Dirac(g, 1.0, 0.1)
D.update(A)
b = rand_spinor(rng, g.n_sites)
h = hashlib.sha256()
for op in (0, 1, 2):
    x, it, ok = D.bicgstab(b, op, tol=1e-10)
    h.update(x.tobytes()); h.update(str((it, ok)).encode())
x, it, _ = D.cg(b, tol=1e-10)
h.update(x.tobytes()); h.update(str(it).encode())
print(h.hexdigest())
"""


def _run(threads):
    env = dict(os.environ, OMP_NUM_THREADS=str(threads))
    out = subprocess.run([sys.executable, "-c", PROG.format(root=ROOT)], env=env, capture_output=True, text=True,
                         timeout=300, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    return out.stdout.strip()


def test_oracle_solvers_independent_of_thread_count():
    ref = _run(1)
    for t in (3, 8):
        assert _run(t) == ref, t
