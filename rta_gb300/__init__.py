"""GB300 (sm_103a) LBVH construction and binary-BVH closest-hit traversal for
rta's bbvh-cuda hot path.

    rta_gb300.lib      ctypes binding of the C ABI (include/rta_gb300.h)
    rta_gb300.plugin   rta's plugin interfaces (constructor, tracers, rays,
                       bouncers, create_rt_set) over that ABI
    rta_gb300.scenes   seeded synthetic scenes and ray sets
    rta_gb300.build    compiles csrc/*.cu for sm_103a
"""
