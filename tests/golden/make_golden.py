"""Generate the golden fixtures of the CPU oracle (run: python -m tests.golden.make_golden).

Fixtures hold, for small seeded models: dA/dpsi of one EOM evaluation at a
seeded random state and at the single-configuration start, and the observables
of a short propagation (C(t), populations, energy).  They pin the oracle
against regressions; the GPU parity tests compare against the same oracle.
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from macaw_gb300.model import initial_wavefunction  # noqa: E402
from oracle.mctdh import Oracle  # noqa: E402
from tests.helpers import small_lvc, small_qvc, random_state  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))


def compute(name):
    model = {"lvc_small": lambda: small_lvc(tfinal_fs=1.0),
             "qvc_small": lambda: small_qvc(tfinal_fs=0.5)}[name]()
    o = Oracle(model)
    A, psi = random_state(model, seed=42)
    dA, dpsi = o.calc_derivs(A, psi, 0.0)
    A0, psi0 = initial_wavefunction(model)
    dA0, dpsi0 = o.calc_derivs(A0, psi0, 0.0)
    outs, _, _ = o.propagate(A0, psi0)
    return dict(dA=dA, dpsi=dpsi, dA0=dA0, dpsi0=dpsi0,
                t=np.array([r["t"] for r in outs]),
                auto=np.array([r["auto"] for r in outs]),
                pop=np.array([r["pop"] for r in outs]),
                energy=np.array([r["energy"] for r in outs]))


if __name__ == "__main__":
    for name in ("lvc_small", "qvc_small"):
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **compute(name))
        print("wrote", name)
