// life.h — bit-packed, temporally blocked cellular-automaton steps.
#pragma once

#include "dispatch.h"

namespace stc {

// If (stencil, op, boundary, grid) is a 2D Moore(1) outer-totalistic rule on a UInt8/Bool/Int32/Int64
// grid at least 32 cells wide, run as many of `nsteps` as possible on a packed copy and unpack
// the result into the parent the reference's switch() would leave it in.  *done reports how many
// steps ran (0 when the fast path does not apply); *src_is_b is updated accordingly.
int life_try_steps(const stc_grid* a, const stc_grid* b, const stc_stencil* st, const stc_op* op,
                   const stc_bc* bc, int64_t nsteps, int* src_is_b, cudaStream_t stream, DeviceCtx* ctx,
                   int64_t* done);

}  // namespace stc
