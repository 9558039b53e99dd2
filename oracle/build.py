"""Build recipe for the oracle (TEST INFRASTRUCTURE ONLY).

* ``build_oracle()`` compiles oracle/rpm_oracle.cpp (the CPU restatement of the
  reference path) into oracle/_build/librpm_oracle.so.
* ``build_ref()`` compiles the reference's own
  src/state_spaces/real_vector_space/CollisionAndDistance.cpp and
  src/configurations/RealVectorSpaceConfig.cpp, in place from the reference
  tree, against oracle/eigen_standin, into oracle/_ref/libref_cad.so.  It is
  skipped when the reference tree is absent.

Both use ``-ffp-contract=off`` so no multiply-add is fused on any host.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# The reference tree: RPM_REFERENCE_ROOT, else a "reference" directory beside
# this repository.  Where it is absent the reference build is skipped.
REF_ROOT = os.environ.get("RPM_REFERENCE_ROOT",
                          os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference"))
ORACLE_SO = os.path.join(HERE, "_build", "librpm_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libref_cad.so")

FLAGS = ["-O2", "-std=c++17", "-shared", "-fPIC", "-ffp-contract=off", "-fno-fast-math"]


def _newer(out, srcs):
    return os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(s) for s in srcs)


def build_oracle(force=False):
    src = os.path.join(HERE, "rpm_oracle.cpp")
    hdr = os.path.join(HERE, "..", "include", "rpm_gpu.h")
    if not force and _newer(ORACLE_SO, [src, hdr]):
        return ORACLE_SO
    os.makedirs(os.path.dirname(ORACLE_SO), exist_ok=True)
    tmp = ORACLE_SO + ".tmp%d" % os.getpid()
    subprocess.check_call(["g++", *FLAGS, "-fopenmp", src, "-o", tmp])
    os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def build_ref(force=False):
    cad = os.path.join(REF_ROOT, "src", "state_spaces", "real_vector_space", "CollisionAndDistance.cpp")
    cfg = os.path.join(REF_ROOT, "src", "configurations", "RealVectorSpaceConfig.cpp")
    if not (os.path.exists(cad) and os.path.exists(cfg)):
        return None
    wrap = os.path.join(HERE, "ref_wrap.cpp")
    shim = os.path.join(HERE, "eigen_standin", "eigen3", "Eigen", "Dense")
    if not force and _newer(REF_SO, [cad, cfg, wrap, shim]):
        return REF_SO
    os.makedirs(os.path.dirname(REF_SO), exist_ok=True)
    inc = ["-I", os.path.join(HERE, "eigen_standin"),
           "-I", os.path.join(REF_ROOT, "include", "state_spaces", "real_vector_space"),
           "-I", os.path.join(REF_ROOT, "include", "configurations")]
    tmp = REF_SO + ".tmp%d" % os.getpid()
    subprocess.check_call(["g++", *FLAGS, "-w", *inc, cad, cfg, wrap, "-o", tmp])
    os.replace(tmp, REF_SO)
    return REF_SO


if __name__ == "__main__":
    print(build_oracle(force="-f" in sys.argv))
    print(build_ref(force="-f" in sys.argv))
