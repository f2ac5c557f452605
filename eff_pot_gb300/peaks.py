"""Measure the FMA throughput of this GPU (FP64 and FP32), the denominator of
the FP64 ALU roofline reported beside the HBM one.

    python -m eff_pot_gb300.peaks          # prints {"fp64_tflops": ..., ...}
"""
import json
import os
import subprocess

from .build import ARCH, BUILD, nvcc

HERE = os.path.dirname(os.path.abspath(__file__))


def measure():
    src = os.path.join(HERE, "csrc", "ep_fma_peak.cu")
    exe = os.path.join(BUILD, "fma_peak")
    os.makedirs(BUILD, exist_ok=True)
    subprocess.check_call([nvcc(), "-O3", "-std=c++17"] + ARCH + [src, "-o", exe])
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    return json.loads(out.strip().splitlines()[-1])


if __name__ == "__main__":
    print(json.dumps(measure()))
