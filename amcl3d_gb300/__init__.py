"""amcl3d_gb300: the particle-filter hot path of amcl3d on one GB300 GPU.

``Grid3d`` and ``ParticleFilter`` mirror the reference's classes and ``VoxelGrid``
the scan filter its node applies first; every call runs
in the CUDA library ``_lib/libamcl3d_gpu.so`` (C ABI: ``include/amcl3d_gpu.h``).
Attributes load the library on first use, so ``amcl3d_gb300.build`` can run
before the library exists.
"""

__all__ = ["Grid3d", "ParticleFilter", "Particle", "VoxelGrid"]


def __getattr__(name):
    if name in __all__:
        from . import filter as _f

        return getattr(_f, name)
    raise AttributeError(name)
