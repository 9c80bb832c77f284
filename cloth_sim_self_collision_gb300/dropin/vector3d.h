// vector3d.h -- drop-in replacement of the reference header of the same name: the
// CVector3D point type of the distance and coplanarity functions (bvh_aabb.h) is
// declared in clothgpu_dropin.h.
#include "clothgpu_dropin.h"
