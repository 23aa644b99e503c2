// Run-time specialized passes (csrc/jit.cu): host interface.
#pragma once

#include <memory>
#include <string>
#include <vector>

#include "common.cuh"
#include "program.cuh"

namespace lsg {

// Threads of a pipelined pass CTA (256 compute threads and the producer warp; tile.cuh).
constexpr int kPipeThreadsHost = 288;

// The compiled kernels of one program's passes (CUfunction handles, one per pass).
// The modules are unloaded with the last reference (the cache's or a program's; a program is
// destroyed only after its kernels finished).
struct JitPasses {
    std::vector<void*> fns;      // CUfunction per pass
    std::vector<int> per_sm;     // resident CTAs per SM of each pass at its shared memory
    bool swz = false;            // tiles move by swizzled tensor copies (common.cuh Tmap)
    std::vector<void*> modules;  // CUmodule per compiled unit
    JitPasses() = default;
    JitPasses(const JitPasses&) = delete;
    JitPasses& operator=(const JitPasses&) = delete;
    ~JitPasses();
};

// LSG_JIT: 0 never specialize, 1 always, unset: programs whose one run moves at least
// LSG_JIT_MIN_BYTES of HBM traffic (default 256 GiB, about 0.15 s interpreted, where the second or
// so of compilation is recovered within a few dozen runs).
int jit_mode();
bool jit_wanted(int64_t bytes_per_run);
// Whether real32 group pairs run as packed 64-bit operands (fma.rn.f32x2; LSG_FFMA2=0: never).
bool jit_packed(int precision);

// The CUDA source of a planned gate program's specialized passes, or "" when a pass can't be.
std::string jit_source(const Plan& plan, int precision, int ctas, bool swz, bool packed);

// Compile `source` with NVRTC only (no device needed): LSG_OK, or an error with NVRTC's log.
int jit_compile_check(const std::string& source);

// Whether a program's specialized passes can move tiles as tensor boxes with the 128-byte swizzle:
// every pass's contiguous chunks are 512 bytes (moved in pairs across register bit hi[0]) or whole
// 1 KB swizzle atoms, and the register's 128-byte rows fit 31-bit coordinates.
bool jit_swizzle_fits(const Plan& plan, size_t elem_bytes, int64_t register_bytes);

// Specialize a planned gate program (no trajectory operators, no shared-memory operators), or
// nullptr when it can't be (unsupported operators, no NVRTC, compilation failure): the
// interpreter then runs it. `ctas` is the launch bound's CTAs per SM. Passes compile in parallel
// on host threads; modules are cached by plan (the descriptors the source is generated from) for
// the life of the process, so a program of a known shape generates no source.
std::shared_ptr<JitPasses> jit_build(const Plan& plan, int precision, int ctas, bool swz, bool packed);

// Launch every pass on `stream` (events before each pass when `marks` is given).
// `tiles_per_member[i]`: the tiles pass i visits in each of the `batch` members.
int jit_launch(const JitPasses& jp, const Plan& plan, void* state, int64_t member_elems, const void* pass_dev,
               size_t pass_stride, const void* data, const std::vector<int64_t>& tiles_per_member, int64_t batch,
               int* status, size_t tile_bytes, cudaStream_t stream, cudaEvent_t* marks);

}  // namespace lsg
