"""arborx_gb300 -- GB300-native (sm_103a) ArborX BoundingVolumeHierarchy.

Python face of the C ABI in include/arborx_gb300.h, shaped like ArborX's
API (src/spatial/ArborX_LinearBVH.hpp, ArborX_CrsGraphWrapper.hpp):

    bvh = BoundingVolumeHierarchy(points)              # torch cuda [n,3] f32
    indices, offsets = query(bvh, make_intersects(centres, r))
    indices, offsets = query(bvh, make_nearest(points, k),
                             TraversalPolicy().setPredicateSorting(False))

All compute runs in libarborx_gb300.so; tensors are passed as raw device
pointers and results are zero-copy views of the library's own buffers.
"""

from ._lib import BOX, KDOP6, KDOP14, KDOP18, KDOP26, POINT, RAY, SPHERE, AbxError, SearchException  # noqa: F401
from .serve import Server  # noqa: F401
from .bvh import (  # noqa: F401
    BoundingVolumeHierarchy,
    BruteForce,
    Forest,
    Intersects,
    Nearest,
    TraversalPolicy,
    device_errors,
    exclusive_scan,
    expand_half_to_full,
    find_full_neighbor_list,
    find_half_neighbor_list,
    generate_hierarchy,
    intersects,
    kdop_from,
    make_intersects,
    make_nearest,
    morton32,
    morton64,
    nearest,
    ordered_intersects,
    ray_intersects,
    query,
    query_nearest_host,
    query_nearest_into,
    scene_bounds,
    sort_u32,
    sort_u64,
    version,
)

BVH = BoundingVolumeHierarchy
