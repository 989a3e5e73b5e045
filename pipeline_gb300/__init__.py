"""pipeline_gb300: GB300-native (sm_103a) octree construction.

A drop-in for the seven-stage octree build of ucsc-redwood/pipeline (Morton
encode, radix sort, unique, Karras radix tree, edge count, prefix sum, octree
nodes + leaf links). The compute path is the native library
``_lib/libpipeline_gb300.so`` (C ABI in include/octree_gb300.h); this package
is its host-side mirror:

  kernels   the reference's per-stage functions (k_ComputeMortonCode, ...)
            on CUDA tensors
  pipeline  OctreeBuilder: the whole build with device-resident sizes,
            CUDA-graph capturable
  datasets  seeded synthetic clouds (uniform, clustered, batched, scan frames)
"""
from ._lib import OCT_MAX_N, OctError, load  # noqa: F401

__all__ = ["OCT_MAX_N", "OctError", "load"]
