"""fluidsim_gb300: the per-step hot path of fluidsim's 2D argon
drift-diffusion discharge on one GB300 (C ABI in include/fluidsim_gpu.h,
Python front end in api.py)."""
import os

# Every context runs on its own CUDA stream and the batch driver keeps many in
# flight; with the default 8 hardware work queues their kernels serialise
# (a 192-discharge sweep: 1397 against 1910 steps/s with 32 queues).  The
# setting takes effect only if it is in place before the process creates its
# CUDA context, and a value the user set is kept.
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
