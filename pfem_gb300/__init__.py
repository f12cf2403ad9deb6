"""GB300-native PFEM per-time-step solve.

* `pfem_gb300.api`   - ctypes binding of the C ABI (include/pfem_gpu.h, libpfemgpu.so)
* `pfem_gb300.mesh`  - host-side node clouds and alpha-shape triangulation
* `pfem_gb300.solver` - host mirror of the reference's Solver classes (time loop, remesh, dt)
* `pfem_gb300.build` - builds libpfemgpu.so with nvcc for sm_103a
"""
__version__ = "0.1.0"
