// Launchers of the tile-pass kernels. Each element type's kernels are instantiated in a
// translation unit of their own (kernels_<type>.cu), so the build compiles them in parallel; the
// host code (engine.cu) reaches them only through these functions.
#pragma once

#include "tile.cuh"

namespace lsg {

template <typename T>
struct PassKernels {
    // the kernels, for attribute and occupancy queries
    static const void* pipe();
    static const void* pass();
    static const void* ragged();
    // k_tile_pipe<T> with kPipeThreads threads, k_tile_pass<T> with 256, k_tile_pipe_ragged<T>
    static void launch_pipe(unsigned grid, size_t smem, cudaStream_t st, T* state, int64_t member_elems,
                            const PassDesc* pass, const TileOp* ops, const BlockDesc* blocks, const T* data,
                            int64_t tiles_per_member, int64_t total_tiles, int* status, const TrajCtx& ctx);
    static void launch_pass(unsigned grid, size_t smem, cudaStream_t st, T* state, int64_t member_elems,
                            const PassDesc* pass, const TileOp* ops, const BlockDesc* blocks, const T* data,
                            int64_t tiles_per_member, int64_t total_tiles, int* status, const TrajCtx& ctx);
    static void launch_ragged(unsigned grid, size_t smem, cudaStream_t st, const RaggedJob* jobs, int njobs, int* status);
};

}  // namespace lsg
