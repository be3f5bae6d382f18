"""Build of the C host program tests/c_driver/step_driver.c with gcc
against include/gmcore_gpu.h, linked to the in-tree library."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "c_driver", "step_driver.c")
LIBDIR = os.path.join(ROOT, "gmcore_gb300", "lib")


def build(outdir):
    from gmcore_gb300 import load
    load()   # builds the library in-tree when it is missing
    exe = os.path.join(outdir, "step_driver")
    cmd = ["gcc", "-std=c99", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), SRC,
           "-L", LIBDIR, "-lgmcore_gpu", "-Wl,-rpath," + LIBDIR, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("step_driver build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return exe
