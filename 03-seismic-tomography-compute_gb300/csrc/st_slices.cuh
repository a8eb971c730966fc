// Internal interface of the slice stream (st_slices.cu) for the solver's
// RTM loop.
#pragma once

#include "st_common.cuh"

namespace stg {

// Sources of one slice capture: forward and adjoint fields (device layout
// FP32 or reference layout FP64; null = zeros) or, for the forward field, a
// compact interior snapshot with its |max| scale word; the image condition
// as an FP32 / FP64 interior array (null = zeros).
struct SliceSrc {
    const void* fwd;
    const void* adj;
    const void* ic;
    int field_kind, ic_kind;
    Layout L;
    int fwd_snap = SNAP_NONE;
    const unsigned* fwd_amax = nullptr;
};

// Enqueues one frame per spec of the stream on `st`.
int slice_stream_capture(st_slice_stream* ss, const SliceSrc& S, int64_t timestep, cudaStream_t st);
// Grid extents the stream was created for.
void slice_stream_extents(const st_slice_stream* ss, int64_t* nx, int64_t* ny, int64_t* nz);

}  // namespace stg
