"""Parity oracle for the descent time step -- TEST INFRASTRUCTURE ONLY.

Two checkers live here, and nothing in the product path imports them:

* ``oracle.restated`` -- ctypes binding of ``phybs_oracle.cpp``, a C++
  restatement of the reference's CPU solver templated on float/double
  (FP32 parity and the all-FP64 reference).  Built by :func:`build`.
* ``oracle.ref`` -- ctypes binding of ``_ref/libphybs_ref.so``, the reference's
  own CPU solver compiled headless from the reference sources
  (``ref_build/Makefile``).  Only buildable where the reference tree exists;
  its outputs are frozen into ``tests/golden`` for everywhere else.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libphybs_ref.so")
# The reference checkout (the directory holding FVM/ and model/): required
# for building oracle/_ref and for the tests that read the reference's own
# files; unset, those are skipped.
REFERENCE_TREE = os.environ.get("PHYBS_REFERENCE") or None


def reference_tree():
    """The reference checkout named by PHYBS_REFERENCE, or None when it is
    unset or lacks FVM/."""
    t = os.environ.get("PHYBS_REFERENCE") or REFERENCE_TREE
    return t if t and os.path.isdir(os.path.join(t, "FVM")) else None


def build(reference: bool = True, verbose: bool = False) -> None:
    """Compile the restated oracle; also the reference harness when the
    reference tree (PHYBS_REFERENCE) is present."""
    src = os.path.join(HERE, "phybs_oracle.cpp")
    if (not os.path.exists(ORACLE_SO)) or os.path.getmtime(ORACLE_SO) < os.path.getmtime(src):
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-o", ORACLE_SO, src]
        # OpenMP only parallelises the per-tet loops (results are identical);
        # without it the oracle builds serial
        r = subprocess.run(cmd[:1] + ["-fopenmp"] + cmd[1:], capture_output=True)
        if r.returncode != 0:
            subprocess.run(cmd, check=True, capture_output=not verbose)
    tree = reference_tree()
    if reference and tree:
        subprocess.run(["make", "-s", "-C", os.path.join(HERE, "ref_build"), f"REF={tree}", "-j8"],
                       check=True, capture_output=not verbose)
