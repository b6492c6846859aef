"""skewengine_gb300: GB300-native skewed-data-mapping engine.

For every angle the engine skews a 2-D grid so lines at that angle become memory
rows, runs a per-row operator (total viewshed, Radon / filtered back-projection,
local Radon transform, cepstrum blur estimation, identity), deskews the result and accumulates it.  The
compute runs as hand-written sm_103a CUDA kernels behind the C ABI in
``include/skewengine.h``; this package is its Python host interface.
"""
from .engine import (ACCUM_KAHAN, ACCUM_REFERENCE, DEFAULT_POVH, FLAG_CEPSTRUM_F32, FLAG_LOCAL_RADON_F32, FLAG_NO_GRAPH, FLAG_RADON_F32, FLAG_NO_TUNE, KERNEL_CEPSTRUM,
                     KERNEL_IDENTITYDEM,
                     KERNEL_IDENTITYIMG, KERNEL_LOCAL_RADON, KERNEL_RADON, KERNEL_SDEM, KERNELS, SkewEngine,
                     cli_run, device_count, execute, geometry, params, png_size, read_grid, read_image, read_png_rgba,
                     render, render_input, run_batch, write_png)
from ._lib import SkeError

__all__ = ["SkewEngine", "SkeError", "execute", "run_batch", "geometry", "params", "device_count", "cli_run",
           "png_size", "read_grid", "read_png_rgba", "read_image", "write_png", "render", "render_input",
           "KERNEL_SDEM", "KERNEL_IDENTITYDEM", "KERNEL_RADON", "KERNEL_IDENTITYIMG", "KERNEL_CEPSTRUM",
           "KERNEL_LOCAL_RADON",
           "KERNELS", "ACCUM_REFERENCE", "ACCUM_KAHAN", "DEFAULT_POVH", "FLAG_NO_TUNE", "FLAG_NO_GRAPH", "FLAG_CEPSTRUM_F32",
           "FLAG_LOCAL_RADON_F32", "FLAG_RADON_F32"]
