"""GB300-native (sm_103a) path tracer with HastyRenderer's render-job surface.

The compute path is CUDA behind the C ABI in include/hasty_gpu.h; this package
holds the ctypes binding (`native`), a Python mirror of the reference's job
interface (`api`), the in-tree build (`build`) and seeded scene generators
(`scenes`).
"""
from .api import (AOV_ALBEDO, AOV_COLOR, AOV_NORMAL, Context, HastyError, RenderJob, Server, batch_render,  # noqa: F401
                  debug_bsdf, load_jobs)

__version__ = "0.1.0"
