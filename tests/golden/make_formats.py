"""Generates tests/golden/ref_written.npz: text files written by the psvWave
reference's own solver (oracle/_ref/libpsv_ref.so, built from the reference
sources by oracle/build_ref.sh), for the cross-implementation file-format
tests. Run from the repository root:

    python oracle/build.py && python tests/golden/make_formats.py

The run is the small golden configuration (tests/golden/small.ini) with the
golden target and start media: observed data from the target, then one
gradient at the start medium (src/psvWave.cpp:518-545 call order). Files
(each stored as its bytes under its file name):
  rtf_ux{0,1}.txt, rtf_uz{0,1}.txt -- write_receivers: the start medium's
      seismograms, 25 significant digits (src/fdModel.cpp:971-1006);
  sources_shot_{0,1}.txt -- write_sources (src/fdModel.cpp:1008-1032);
  kernel_vp.txt, kernel_vs.txt, kernel_density.txt -- write_kernels
      (src/fdModel.cpp:1326-1356);
  snapshots/v{x,z}00{100,300}.txt -- wave-field dumps of a forward run of
      shot 0 (src/fdModel.cpp:753-776), two of its instants;
  model_vector.txt -- a model vector file (3 nx_free nz_free seeded values,
      written with 17 significant digits) that the reference's load_vector
      reads (src/fdModel.cpp:1517-1572); `loaded_vector` holds what it read.
"""
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import refbind  # noqa: E402

SMALL_INI = os.path.join(HERE, "small.ini")
DUMPS = ("snapshots/vx00100.txt", "snapshots/vz00100.txt", "snapshots/vx00300.txt",
         "snapshots/vz00300.txt")


def gradient(m, target, start):
    m.set_parameter_fields(*target)
    for s in range(m.n_shots):
        m.forward_simulate(s, True)
    m.set_observed_data(*m.get_synthetic_data())
    m.set_parameter_fields(*start)
    for s in range(m.n_shots):
        m.forward_simulate(s, True)
    m.calculate_l2_misfit()
    m.calculate_l2_adjoint_sources()
    m.reset_kernels()
    for s in range(m.n_shots):
        m.adjoint_simulate(s)
    m.map_kernels_to_velocity()


def vector_file_values(m):
    """3 nx_free nz_free values: the count the reference's load_vector reads
    (one per free cell and parameter, whatever the basis blocks)."""
    rng = np.random.default_rng(21)
    n = m.info["nx_free_parameters"] * m.info["nz_free_parameters"]
    base = np.repeat([2000.0, 800.0, 1500.0], n)
    return base * (1.0 + 0.01 * rng.standard_normal(3 * n))


def main():
    golden = dict(np.load(os.path.join(HERE, "small_golden.npz")))
    out = {}
    cwd = os.getcwd()
    with tempfile.TemporaryDirectory() as tmp:
        os.chdir(tmp)
        try:
            os.makedirs("snapshots")
            m = refbind.RefModel(SMALL_INI)
            gradient(m, tuple(golden["target"]), tuple(golden["start"]))
            m.write_receivers()
            m.write_sources()
            m.write_kernels()
            m.forward_simulate_output(0, False)
            np.savetxt("model_vector.txt", vector_file_values(m), fmt="%.17g")
            out["loaded_vector"] = m.load_vector(os.path.join(tmp, "model_vector.txt"))
            names = (["rtf_ux%d.txt" % s for s in range(m.n_shots)] +
                     ["rtf_uz%d.txt" % s for s in range(m.n_shots)] +
                     ["sources_shot_%d.txt" % s for s in range(m.n_shots)] +
                     ["kernel_vp.txt", "kernel_vs.txt", "kernel_density.txt",
                      "model_vector.txt"] + list(DUMPS))
            for n in names:
                with open(n, "rb") as f:
                    out["file:" + n] = np.frombuffer(f.read(), dtype=np.uint8)
        finally:
            os.chdir(cwd)
    path = os.path.join(HERE, "ref_written.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
