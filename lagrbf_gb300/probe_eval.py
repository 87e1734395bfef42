"""Compute-only bound of the FP32 evaluation's record loop on the current GPU.

Builds lagrbf_gb300/csrc/probe_record_loop.cu (nvcc, sm_103a; not part of liblagrbf.so), measures
the FFMA peak with the library's probe, and runs the loop body with records resident in shared
memory for one and two particle pairs per thread: the ceiling that staging, prologue and epilogue
of k_eval_rec are compared against.

    python -m lagrbf_gb300.probe_eval
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc", "probe_record_loop.cu")
EXE = os.path.join(HERE, "_build", "probe_record_loop")


def main():
    from lagrbf_gb300 import build
    cuda = build._cuda_home()
    os.makedirs(os.path.dirname(EXE), exist_ok=True)
    subprocess.run([os.path.join(cuda, "bin", "nvcc"), "-O3", "-std=c++17", *build.ARCH, SRC, "-o", EXE], check=True)
    from lagrbf_gb300._lib import load_cfuncs
    peak = load_cfuncs()["lagrbf_gpu_fp32_peak_tflops"]()
    print("FFMA peak (library probe): %.1f TFLOP/s" % peak, flush=True)
    return subprocess.run([EXE, "%.3f" % peak]).returncode


if __name__ == "__main__":
    sys.exit(main())
