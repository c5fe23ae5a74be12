"""Build recipe for the oracle (test infrastructure only).

* oracle/_build/libpsv_oracle.so -- the C restatement (psv_oracle.c), built
  everywhere, with -ffp-contract=off so that no multiply-add is fused and
  the arithmetic stays bit-identical to the reference's double code on both
  x86-64 and aarch64 hosts.
* oracle/_ref/libpsv_ref.so -- the reference's own solver sources, built by
  build_ref.sh only where those sources are present.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
PORT_LIB = os.path.join(BUILD, "libpsv_oracle.so")


def build_port(force=False):
    src = os.path.join(HERE, "psv_oracle.c")
    hdr = os.path.join(HERE, "psv_oracle.h")
    if (not force and os.path.exists(PORT_LIB)
            and os.path.getmtime(PORT_LIB) >= max(os.path.getmtime(src), os.path.getmtime(hdr))):
        return PORT_LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = PORT_LIB + ".tmp"
    subprocess.check_call(["gcc", "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
                           "-std=c99", "-Wall", "-Wno-unused-result", "-Wno-format-truncation", src, "-o", tmp, "-lm"])
    os.replace(tmp, PORT_LIB)
    return PORT_LIB


# Where the reference checkout's sources lie on the machine that made the
# fixtures (read-only there); REF_SRC overrides it. Machines without the
# checkout (the GPU hosts) skip the reference build.
REF_CHECKOUT_SRC = "/root/reference/src"


def ref_src():
    return os.environ.get("REF_SRC", REF_CHECKOUT_SRC)


def build_ref():
    env = dict(os.environ, REF_SRC=ref_src())
    subprocess.check_call(["sh", os.path.join(HERE, "build_ref.sh")], env=env)


def build_all():
    build_port()
    if os.path.isfile(os.path.join(ref_src(), "fdModel.cpp")):
        build_ref()


if __name__ == "__main__":
    build_all()
    sys.exit(0)
