"""ctypes access to the FP64 CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
this module.  The oracle exports the C ABI of include/filament_gb.h with the
symbol prefix "filo_", so the same host driver runs against it.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libfil_oracle.so")


def build(quiet=True):
    r = subprocess.run(["make", "-C", HERE], capture_output=quiet, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n%s%s" % (r.stdout or "", r.stderr or ""))
    return LIB


def binding():
    import filament_gb._abi as abi
    if not os.path.exists(LIB):
        build()
    return abi.Binding(LIB, "filo_")
