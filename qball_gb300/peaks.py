"""Measure the FP64/FP32 arithmetic peaks used as roofline denominators.

    python -m qball_gb300.peaks

Compiles csrc/peaks_probe.cu for sm_103a into _build/ and runs it on GPU 0.
"""
import os
import subprocess
import sys

from qball_gb300 import build as B


def main():
    os.makedirs(B.BUILD, exist_ok=True)
    exe = os.path.join(B.BUILD, "peaks_probe")
    subprocess.run([B.nvcc(), *B.ARCH, "-O3", os.path.join(B.CSRC, "peaks_probe.cu"), "-o", exe],
                   check=True)
    return subprocess.run([exe]).returncode


if __name__ == "__main__":
    sys.exit(main())
