// self_collision_cloth.h -- drop-in replacement of the reference header of the same name: the
// declarations the self_contact_sparse driver uses, run on the GPU (clothgpu_dropin.h).
#include "clothgpu_dropin.h"
