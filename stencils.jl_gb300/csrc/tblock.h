// tblock.h — temporally blocked multi-step maps on 3D grids (see tblock3d.cu).
#pragma once

#include "dispatch.h"

namespace stc {

// If the run qualifies (3D grid, radius-1 registered shape, float state, Wrap or Remove, TMA-aligned
// parents), advance nsteps-1 steps with the temporally blocked kernel, leaving state nsteps-1 in the
// parent where the reference's loop leaves it; the caller runs the last step with the per-step map.
// *done reports the steps run (0 when the path does not apply).
int tb3d_try_steps(const stc_grid* a, const stc_grid* b, const stc_stencil* st, const stc_op* op,
                   const stc_bc* bc, int64_t nsteps, int* src_is_b, cudaStream_t stream, DeviceCtx* ctx,
                   int64_t* done);

}  // namespace stc
