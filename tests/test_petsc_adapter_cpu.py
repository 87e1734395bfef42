"""Compile check of the in-process GPU plug-ins (lagrbf_gb300/adapters/petsc) against LagRBF's own,
unchanged headers: every plug-in has the signature of the reference plug-in point it replaces
(RBFInterpolation, SwarmInterpSetWeights, PartitionOfUnity->psetup/psolve/pdestroy,
AdvectionCtx->advection), checked by the compiler through the reference prototypes and the struct
fields the plug-ins are assigned to; every C-ABI call they make is declared in include/lagrbf.h.
PETSc itself is replaced by the stand-in header of oracle/ref_pin (declarations only).  Needs the
LagRBF source tree (LAGRBF_REFERENCE); skipped without it."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "lagrbf_gb300", "adapters", "petsc", "lagrbf_petsc_gpu.c")


def _compile(tmp_path, *defs, extra=None):
    ref = os.environ.get("LAGRBF_REFERENCE")
    if not ref or not os.path.isdir(os.path.join(ref, "include")):
        pytest.skip("LAGRBF_REFERENCE (a LagRBF checkout) not set")
    if not shutil.which("gcc"):
        pytest.skip("no gcc")
    src = SRC
    if extra:
        src = str(tmp_path / "check.c")
        with open(src, "w") as f:
            f.write('#include "%s"\n%s\n' % (SRC, extra))
    cmd = ["gcc", "-std=gnu11", "-c", "-Wall", "-Werror=incompatible-pointer-types",
           "-Werror=implicit-function-declaration", "-I", os.path.join(ROOT, "oracle", "ref_pin"),
           "-I", os.path.join(ref, "include"), "-I", os.path.join(ROOT, "include"),
           "-I", os.path.dirname(SRC), *defs, src, "-o", str(tmp_path / "a.o")]
    return subprocess.run(cmd, capture_output=True, text=True)


def test_plugins_compile_against_reference_headers(tmp_path):
    r = _compile(tmp_path)
    assert r.returncode == 0, r.stderr
    r = _compile(tmp_path, "-DLAGRBF_GPU_REPLACE")  # defined under the reference names
    assert r.returncode == 0, r.stderr


def test_a_wrong_signature_is_rejected(tmp_path):
    """The check is live: a plug-in with another signature does not compile into the slot."""
    bad = ("static PetscErrorCode bad(LagRBFCtx c, Partition p) { return 0; }\n"
           "void f(PartitionOfUnity pu) { pu->psetup = bad; }\n")
    r = _compile(tmp_path, extra=bad)
    assert r.returncode != 0 and "incompatible" in r.stderr
