// tblock.h — temporally blocked multi-step maps: 3D grids (tblock3d.cu) and 2D Float32 grids (tblock2d.cu).
#pragma once

#include "dispatch.h"

namespace stc {

// True if the blocked kernel is compiled for (grid, stencil, op, boundary): a 3D grid, a radius-1
// VonNeumann / Cross table with a registered float op, Wrap or Remove.
bool tb3d_applies(const stc_grid* a, const stc_stencil* st, const stc_op* op, const stc_bc* bc);

// If the run qualifies, advance all nsteps on an internal padded pair (blocked passes of 4 steps, the
// last 1 to 4 steps as per-step maps) and copy states n and n - 1 to the parents where the reference's
// loop leaves them.  *done reports the steps run (0 when the path does not apply); with STC_KEEP_F32
// in `flags` a run the path cannot take returns STC_ERR_UNSUPPORTED instead.
int tb3d_try_steps(const stc_grid* a, const stc_grid* b, const stc_stencil* st, const stc_op* op,
                   const stc_bc* bc, int64_t nsteps, int* src_is_b, cudaStream_t stream, DeviceCtx* ctx,
                   uint32_t flags, int64_t* done);

// True if the 2D blocked kernel is compiled for (grid, stencil, op, boundary): a 2D Float32 grid, a
// radius-1 Window / Moore / VonNeumann table with the mean or sum fold (or diffusion on VonNeumann),
// Wrap or Remove.
bool tb2d_applies(const stc_grid* a, const stc_stencil* st, const stc_op* op, const stc_bc* bc);

// If the run qualifies, advance an even number of blocked passes of K (8) steps, each reading one parent
// and writing the other, leaving at least one step.  *done reports the steps run (0 when the path does
// not apply) and *src_is_b where the latest state is; the caller runs the remaining 1 to 2K steps as
// per-step maps, which leaves state n where the reference's loop does.
int tb2d_try_steps(const stc_grid* a, const stc_grid* b, const stc_stencil* st, const stc_op* op,
                   const stc_bc* bc, int64_t nsteps, int* src_is_b, cudaStream_t stream, DeviceCtx* ctx,
                   int64_t* done);

}  // namespace stc
