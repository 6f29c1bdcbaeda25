"""Build recipe for the CPU oracle (test infrastructure only).

* ``oracle/liboracle.so``   -- the C restatement (orc_constitutive.c, orc_problem.c)
* ``oracle/_ref/libipfem_ref.so`` -- the reference's own constitutive headers
  (FunctionsStressStrain.h, FunctionsTangentOperator.h, compiled unmodified from
  the reference tree named by IPFEM_REFERENCE_DIR, by default the directory
  `reference` beside the repository root)
  behind oracle/ref_driver.cpp and the two-header shim in oracle/ref_shim/.
  Built only where the reference tree exists; outputs go to oracle/_ref/ only.

Flags: -ffp-contract=off keeps every multiply and add separately rounded, as in
the reference's x86-64 CPU build (no FMA instructions at the baseline ISA);
-ftrivial-auto-var-init=zero gives the reference's uninitialised gamma[2]
(FunctionsSigmaProjection.h:103, 205) the value 0.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")
REF_SO = os.path.join(REF_DIR, "libipfem_ref.so")
ORACLE_SRC = ["orc_constitutive.c", "orc_problem.c"]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build_oracle(force=False):
    srcs = [os.path.join(HERE, s) for s in ORACLE_SRC]
    deps = srcs + [os.path.join(HERE, h) for h in ("ipfem_oracle.h", "orc_problem.h")]
    if force or _stale(ORACLE_SO, deps):
        tmp = ORACLE_SO + ".tmp%d" % os.getpid()
        cmd = ["gcc", "-std=gnu11", "-O2", "-fPIC", "-shared", "-ffp-contract=off",
               "-fno-math-errno", "-fopenmp", "-Wall", "-o", tmp] + srcs + ["-lm"]
        subprocess.check_call(cmd)
        os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def reference_dir():
    """the reference tree: IPFEM_REFERENCE_DIR, else `reference` beside the
    repository root (absent on machines that only run the prebuilt files)"""
    d = os.environ.get("IPFEM_REFERENCE_DIR")
    if d:
        return d
    return os.path.normpath(os.path.join(HERE, "..", "..", "reference"))


def build_ref(force=False):
    """Compile the reference constitutive headers; returns the .so path or None
    when the reference tree is not present on this machine."""
    rdir = reference_dir()
    hdr = os.path.join(rdir, "FunctionsStressStrain.h")
    if not os.path.exists(hdr):
        return None
    os.makedirs(REF_DIR, exist_ok=True)
    drv = os.path.join(HERE, "ref_driver.cpp")
    deps = [drv, hdr, os.path.join(HERE, "ref_shim", "pzreal.h"), os.path.join(HERE, "ref_shim", "TPZTensor.h")]
    if force or _stale(REF_SO, deps):
        tmp = REF_SO + ".tmp%d" % os.getpid()
        cmd = ["g++", "-std=c++14", "-O2", "-fPIC", "-shared", "-ffp-contract=off",
               "-ftrivial-auto-var-init=zero", "-w",
               "-I" + os.path.join(HERE, "ref_shim"), "-I" + rdir, drv, "-o", tmp]
        subprocess.check_call(cmd)
        os.replace(tmp, REF_SO)
    return REF_SO


def build_all(force=False):
    return build_oracle(force), build_ref(force)


if __name__ == "__main__":
    print(build_all(force="--force" in sys.argv))
