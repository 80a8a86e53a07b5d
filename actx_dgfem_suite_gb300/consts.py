"""Device peaks for the roofline, mirroring ``actx_dgfem_suite/consts.py:1-12``.

The reference's table holds datasheet FP64 and bandwidth figures for Titan V
and H200 NVL.  For GB300 the bandwidth is the measured STREAM-style copy rate
of this deployment's GPUs; the FP64 rate is measured at run time by the
library's FMA probe (``dg_fp64_fma_probe``) because the datasheet figure for
Blackwell Ultra FP64 is far below Hopper's and the roofline depends on it.
"""

# GFLOP/s (FP64) -- datasheet values, as in the reference
DEV_TO_PEAK_F64_GFLOPS = {
    "NVIDIA TITAN V": 6144,
    "NVIDIA H200 NVL": 30000,
    # GB300 (Blackwell Ultra) FP64 datasheet value; bench.py measures it live
    "NVIDIA GB300": 1250,
}

# GB/s
DEV_TO_PEAK_BW = {
    "NVIDIA TITAN V": 652.8,
    "NVIDIA H200 NVL": 4800,
    # measured copy bandwidth (read + write bytes) on this deployment's GB300s
    "NVIDIA GB300": 6791.7,
}
