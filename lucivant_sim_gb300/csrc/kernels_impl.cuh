// Definitions behind kernels.cuh, included by the per-type translation units only.
#pragma once

#include "kernels.cuh"

namespace lsg {

template <typename T>
const void* PassKernels<T>::pipe() {
    return reinterpret_cast<const void*>(k_tile_pipe<T>);
}
template <typename T>
const void* PassKernels<T>::pass() {
    return reinterpret_cast<const void*>(k_tile_pass<T>);
}
template <typename T>
const void* PassKernels<T>::ragged() {
    return reinterpret_cast<const void*>(k_tile_pipe_ragged<T>);
}
template <typename T>
void PassKernels<T>::launch_pipe(unsigned grid, size_t smem, cudaStream_t st, T* state, int64_t member_elems,
                                 const PassDesc* pass, const TileOp* ops, const BlockDesc* blocks, const T* data,
                                 int64_t tiles_per_member, int64_t total_tiles, int* status, const TrajCtx& ctx) {
    k_tile_pipe<T><<<grid, kPipeThreads, smem, st>>>(state, member_elems, pass, ops, blocks, data, tiles_per_member,
                                                     total_tiles, status, ctx);
}
template <typename T>
void PassKernels<T>::launch_pass(unsigned grid, size_t smem, cudaStream_t st, T* state, int64_t member_elems,
                                 const PassDesc* pass, const TileOp* ops, const BlockDesc* blocks, const T* data,
                                 int64_t tiles_per_member, int64_t total_tiles, int* status, const TrajCtx& ctx) {
    k_tile_pass<T><<<grid, 256, smem, st>>>(state, member_elems, pass, ops, blocks, data, tiles_per_member, total_tiles,
                                            status, ctx);
}
template <typename T>
void PassKernels<T>::launch_ragged(unsigned grid, size_t smem, cudaStream_t st, const RaggedJob* jobs, int njobs,
                                   int* status) {
    k_tile_pipe_ragged<T><<<grid, kPipeThreads, smem, st>>>(jobs, njobs, status);
}

}  // namespace lsg
