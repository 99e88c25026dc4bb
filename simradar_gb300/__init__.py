"""simradar_gb300: GB300 (sm_103a) backend for SimRadar's per-pulse emulation loop.

The compute path is libsimradar_gb300.so (CUDA, C ABI in include/rsc.h); the
Python modules here only build it (build.py), bind it (rsc.py) and describe
the synthetic tables and scenes the tests and the benchmark use (synth.py).
"""
import os as _os

LIBRARY_PATH = _os.path.join(_os.path.dirname(_os.path.abspath(__file__)), "lib", "libsimradar_gb300.so")
