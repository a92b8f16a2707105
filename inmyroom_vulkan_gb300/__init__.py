"""GB300-native (sm_103a) collision detection for the inMyRoom_vulkan engine.

The product is the C ABI in ``include/collide_gpu.h`` implemented by
``libcollide_gpu.so`` (CUDA sources in ``csrc/``). Python modules here are thin
host plumbing over that library:

* ``capi``    — ctypes binding of the C ABI (Context, tree upload, collide).
* ``build``   — in-tree nvcc build for sm_103a.
* ``scenes``  — seeded synthetic workloads (rigid pair, scene, batch sweep).
"""
__all__ = ["capi", "build", "scenes"]
