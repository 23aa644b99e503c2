// Shared definitions for the engine: error reporting across the C ABI, the register handle,
// complex arithmetic in two precisions, and the inline-PTX primitives (mbarrier, bulk async
// copies) the tile kernels are built on.
#pragma once

#ifndef __CUDACC_RTC__  // (run-time compiled passes see the device parts only)
#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdarg>
#include <cstdio>
#include <string>
#endif

#include "../../include/lsg.h"

namespace lsg {

// ---------------------------------------------------------------- errors across the ABI

int fail(int code, const char* fmt, ...);
void clear_error();

#define LSG_CUDA(call)                                                                          \
    do {                                                                                        \
        cudaError_t e_ = (call);                                                                \
        if (e_ != cudaSuccess)                                                                  \
            return ::lsg::fail(e_ == cudaErrorMemoryAllocation ? LSG_E_MEMORY : LSG_E_CUDA,     \
                               "%s failed: %s", #call, cudaGetErrorString(e_));                 \
    } while (0)

#define LSG_CHECK(status)          \
    do {                           \
        int s_ = (status);         \
        if (s_ != LSG_OK) return s_; \
    } while (0)

#ifndef __CUDACC_RTC__
// Device-side status word (one per device, in global memory): kernels that give up on a
// bounded wait record a code there. Read and cleared by check_device_status().
int* device_status();
int check_device_status(cudaStream_t stream);
#endif

// Iteration limit for every spin-wait in the engine's kernels (mbarrier waits). A wait that
// exhausts it records LSG_E_TIMEOUT in g_device_status and the kernel returns early.
constexpr long long kSpinLimit = 1ll << 28;

constexpr int kMaxBits = 26;  // 2^26 amplitudes per member (Orrery's statevector guard)

#ifndef __CUDACC_RTC__
// ---------------------------------------------------------------- register handle

// A device buffer that grows on demand. With a stream it is stream-ordered (cudaMallocAsync /
// cudaFreeAsync): no device-wide synchronisation, so independent registers keep overlapping.
struct Scratch {
    void* ptr = nullptr;
    size_t bytes = 0;
    cudaStream_t stream = nullptr;
};

int ensure(Scratch& s, size_t bytes);
void release(Scratch& s);

}  // namespace lsg

// Bytes per register element: complex128 16, complex64 8, real64 8, real32 4.
inline size_t lsg_elem_bytes(int precision) {
    return precision == LSG_C128 ? 16 : precision == LSG_R32 ? 4 : 8;
}

// Real (Pauli-transfer) register precisions.
inline bool lsg_precision_real(int precision) {
    return precision == LSG_R64 || precision == LSG_R32 || precision == LSG_RD;
}

struct lsg_state_s {
    int nbits = 0;
    int precision = LSG_C128;
    int64_t batch = 1;
    int64_t elems = 1;  // 2^nbits per member
    void* data = nullptr;
    cudaStream_t stream = nullptr;
    lsg::Scratch program;  // uploaded pass programs
    lsg::Scratch scratch;  // reduction partials, CDFs, sampling buffers
    lsg::Scratch scratch2;
    uint64_t uid = 0;  // distinct for every register made in this process (graphs are bound to one)
    size_t elem_bytes() const { return lsg_elem_bytes(precision); }
    bool real() const { return lsg_precision_real(precision); }
    size_t member_bytes() const { return elem_bytes() * (size_t)elems; }
};
#else
}  // namespace lsg
#endif  // !__CUDACC_RTC__

namespace lsg {

// ---------------------------------------------------------------- complex arithmetic

template <typename R>
struct Vec2;
template <>
struct Vec2<double> {
    using T = double2;
};
template <>
struct Vec2<float> {
    using T = float2;
};

template <typename R>
struct Cx {
    R re, im;
    __host__ __device__ Cx() : re(0), im(0) {}
    __host__ __device__ Cx(R r, R i) : re(r), im(i) {}
};

template <typename R>
__device__ __forceinline__ Cx<R> cmul(Cx<R> a, Cx<R> b) {
    return Cx<R>(fma(a.re, b.re, -a.im * b.im), fma(a.re, b.im, a.im * b.re));
}
// acc + a*b
template <typename R>
__device__ __forceinline__ Cx<R> cfma(Cx<R> a, Cx<R> b, Cx<R> acc) {
    acc.re = fma(a.re, b.re, acc.re);
    acc.re = fma(-a.im, b.im, acc.re);
    acc.im = fma(a.re, b.im, acc.im);
    acc.im = fma(a.im, b.re, acc.im);
    return acc;
}

// The same operations on real elements (Pauli-transfer registers), so the tile code is written
// once for an element type T: Cx<float>, Cx<double>, float or double.
__device__ __forceinline__ float cmul(float a, float b) { return a * b; }
__device__ __forceinline__ double cmul(double a, double b) { return a * b; }
__device__ __forceinline__ float cfma(float a, float b, float acc) { return fmaf(a, b, acc); }
__device__ __forceinline__ double cfma(double a, double b, double acc) { return fma(a, b, acc); }

// Double-float elements (LSG_RD registers): a coefficient is the unevaluated sum hi + lo of two
// FP32 words, |lo| <= ulp(hi) / 2: about 48 significant bits. Products and sums run on the FP32
// units with their rounding errors carried exactly (the product's error by a fused multiply-add,
// Dekker 1971; the sum's by Knuth's two-sum, TAOCP vol. 2, 4.2.2), a relative error of about
// 2^-46 per step, where this GPU's FP64 units run at 1/64 of its FP32 rate. The round-to-nearest
// intrinsics keep the compiler from contracting the error terms into other operations.
struct DF {
    float hi, lo;
    __host__ __device__ DF() : hi(0.0f), lo(0.0f) {}
    __host__ __device__ DF(float h, float l) : hi(h), lo(l) {}
    __host__ __device__ explicit DF(double d) : hi((float)d), lo((float)(d - (double)(float)d)) {}
    __host__ __device__ explicit operator double() const { return (double)hi + (double)lo; }
};

// s + e as a normalised pair, for |s| >= |e| (fast two-sum)
__device__ __forceinline__ DF df_norm(float s, float e) {
    const float h = __fadd_rn(s, e);
    return DF(h, __fsub_rn(e, __fsub_rn(h, s)));
}
__device__ __forceinline__ DF cmul(DF a, DF b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);  // the product's rounding error, exactly
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    return df_norm(p, e);
}
// acc + a*b
__device__ __forceinline__ DF cfma(DF a, DF b, DF acc) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    const float s = __fadd_rn(acc.hi, p);  // two-sum of the high parts: s + t = acc.hi + p exactly
    const float v = __fsub_rn(s, acc.hi);
    const float t = __fadd_rn(__fsub_rn(acc.hi, __fsub_rn(s, v)), __fsub_rn(p, v));
    return df_norm(s, __fadd_rn(t, __fadd_rn(e, acc.lo)));
}

// One row of a double-float matrix-vector product: sum over the terms c not marked in `skip`
// of m[c] * a[c]. The high products are summed with two-sums, their rounding errors, the
// products' errors and the cross terms collected in one FP32 word, and the pair renormalised
// once at the end: 4 FP32 instructions for the first term, 12 for each further one, 3 to finish.
template <int N>
__device__ __forceinline__ DF df_dot(const DF* m, const DF* a, unsigned skip) {
    float s = 0.0f, t = 0.0f;
    bool first = true;
#pragma unroll
    for (int c = 0; c < N; ++c) {
        if (skip & (1u << c)) continue;
        const float p = __fmul_rn(m[c].hi, a[c].hi);
        float e = __fmaf_rn(m[c].hi, a[c].hi, -p);
        e = __fmaf_rn(m[c].hi, a[c].lo, e);
        e = __fmaf_rn(m[c].lo, a[c].hi, e);
        if (first) {
            s = p;
            t = e;
            first = false;
        } else {
            const float u = __fadd_rn(s, p);
            const float v = __fsub_rn(u, s);
            const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(u, v)), __fsub_rn(p, v));
            s = u;
            t = __fadd_rn(t, __fadd_rn(err, e));
        }
    }
    return df_norm(s, t);
}

template <typename T>
struct IsDF {
    static constexpr bool value = false;
};
template <>
struct IsDF<DF> {
    static constexpr bool value = true;
};

template <typename T>
struct Elem {  // complex elements
    using R = decltype(T::re);
    static constexpr bool complex = true;
};
template <>
struct Elem<float> {
    using R = float;
    static constexpr bool complex = false;
};
template <>
struct Elem<double> {
    using R = double;
    static constexpr bool complex = false;
};
template <>
struct Elem<DF> {  // FP32 arithmetic: the FP32 register budget and occupancy of 8-byte elements
    using R = float;
    static constexpr bool complex = false;
};

// real part (a real element is its own)
template <typename R>
__host__ __device__ __forceinline__ R re_of(Cx<R> a) {
    return a.re;
}
__host__ __device__ __forceinline__ float re_of(float a) { return a; }
__host__ __device__ __forceinline__ double re_of(double a) { return a; }
__host__ __device__ __forceinline__ float re_of(DF a) { return a.hi; }

// Insert zero bits at the (ascending) positions in `pos` into x: spreads x over the other bits.
__device__ __forceinline__ uint64_t spread(uint64_t x, const int* pos, int k) {
    for (int i = 0; i < k; ++i) {
        uint64_t low = x & ((1ull << pos[i]) - 1);
        x = ((x >> pos[i]) << (pos[i] + 1)) | low;
    }
    return x;
}

// ---------------------------------------------------------------- PTX primitives

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return done != 0;
}

// Bounded wait on an mbarrier phase; false (and a recorded timeout) when the limit is reached.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, int* status) {
    for (long long i = 0; i < kSpinLimit; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    atomicExch(status, LSG_E_TIMEOUT);
    return false;
}

__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Bulk copy global -> shared, completing on an mbarrier (bytes and both addresses 16B aligned).
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

// Bulk copy shared -> global in the current bulk group.
__device__ __forceinline__ void bulk_s2g(void* dst, const void* src, uint32_t bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(smem_u32(src)),
                 "r"(bytes)
                 : "memory");
}

// An encoded tensor map (a CUtensorMap, 128 bytes) for tensor copies, passed to kernels as a
// __grid_constant__ parameter. The register is seen as rows of 128 bytes copied with the 128-byte
// swizzle (16-byte unit u of row r lands at unit u ^ (r & 7), repeating every 1 KB), which spreads
// strided register-block accesses over the shared-memory banks. Every box is a whole number of
// 1 KB swizzle atoms and lands on a 1 KB boundary: a run of rows (2-D map), or two 512-byte chunks
// that differ in one register bit h (3-D map: rows of 128 bytes, blocks of 2^h elements).
struct alignas(64) Tmap {
    unsigned long long w[16];
};

__device__ __forceinline__ void tma_load_2d(void* dst, const Tmap* map, int row, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
        "[%4];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(0), "r"(row), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void tma_load_3d(void* dst, const Tmap* map, int row, int block, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(0), "r"(row), "r"(block), "r"(smem_u32(bar))
        : "memory");
}

// One box shared -> global (un-swizzled back), in the current bulk group.
__device__ __forceinline__ void tma_store_2d(const Tmap* map, int row, const void* src) {
    asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.tile.bulk_group [%0, {%1, %2}], [%3];" ::"l"(
                     reinterpret_cast<uint64_t>(map)),
                 "r"(0), "r"(row), "r"(smem_u32(src))
                 : "memory");
}

__device__ __forceinline__ void tma_store_3d(const Tmap* map, int row, int block, const void* src) {
    asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.tile.bulk_group [%0, {%1, %2, %3}], [%4];" ::"l"(
                     reinterpret_cast<uint64_t>(map)),
                 "r"(0), "r"(row), "r"(block), "r"(smem_u32(src))
                 : "memory");
}

__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }

// Wait until all committed bulk stores have finished reading shared memory.
__device__ __forceinline__ void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
// Wait until all committed bulk stores are complete (visible in global memory).
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

}  // namespace lsg
