"""Generates tests/golden/repo_written.npz on a GPU host: the files this
library's FP64 model writes for the small golden run (the run of
tests/golden/make_formats.py), for the test that has the reference's own
build load them (tests/test_formats.py). Run from the repository root:

    python tests/golden/make_repo_written.py [output.npz]
"""
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import psvwave_gb300 as psv  # noqa: E402
from tests.golden.make_formats import gradient  # noqa: E402


def main(path):
    golden = dict(np.load(os.path.join(HERE, "small_golden.npz")))
    out = {}
    cwd = os.getcwd()
    with tempfile.TemporaryDirectory() as tmp:
        os.chdir(tmp)
        try:
            m = psv.fdModel(os.path.join(HERE, "small.ini"), precision="fp64")
            gradient(m, tuple(golden["target"]), tuple(golden["start"]))
            m.write_receivers()
            m.write_sources()
            for n in sorted(os.listdir(".")):
                with open(n, "rb") as f:
                    out["file:" + n] = np.frombuffer(f.read(), dtype=np.uint8)
            ux, uz = m.get_synthetic_data()
            out["rtf_ux"], out["rtf_uz"] = ux, uz
        finally:
            os.chdir(cwd)
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.join(HERE, "repo_written.npz"))
