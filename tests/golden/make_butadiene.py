"""Fixtures of the reference's two example inputs (run: python -m tests.golden.make_butadiene).

The reference ships two inputs, the 5-mode butadiene model with Gaussian modes
propagated by Dormand-Prince (Examples/Butadiene_5modes) and the same model with
CMF2 (Examples/Butadiene_5modes_CMF).  Their Hamiltonian uses spline-interpolated
potentials ('interp' operators read from data files).  This script reads both
inputs where the reference lies (MACAW_REFERENCE_DIR, default /root/reference)
with this package's parser and stores the declared model -- its constructor
fields, including the data-file points the splines interpolate -- as a pickle
per example, so that the GPU parity tests can run both models where the
reference is absent.  Nothing else of the reference is stored.
"""
import os
import pickle
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from macaw_gb300.model import model_fields, parse_input  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
EXAMPLES = {"butadiene_dopri": "Butadiene_5modes", "butadiene_cmf2": "Butadiene_5modes_CMF"}


def reference_dir() -> str:
    return os.environ.get("MACAW_REFERENCE_DIR", "/root/reference")


def example_input(name: str) -> str:
    return os.path.join(reference_dir(), "Examples", EXAMPLES[name], "but_5D.inp")


def fixture_path(name: str) -> str:
    return os.path.join(HERE, name + ".pkl")


if __name__ == "__main__":
    for name in EXAMPLES:
        model = parse_input(example_input(name))
        with open(fixture_path(name), "wb") as fh:
            pickle.dump(model_fields(model), fh, protocol=4)
        print("wrote", fixture_path(name))
