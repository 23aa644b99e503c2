// Tile-pass device code shared by the gate engine and the trajectory runner: the in-shared-memory
// operators and the fused pass kernel (TMA bulk loads into a 2^K-amplitude tile, every operator
// of the pass, bulk stores back).
#pragma once

#include "common.cuh"
#include "program.cuh"

namespace lsg {

// Per-member context of trajectory runs: each member (shot) reads its uniforms from row
// `member` of `u` starting at `cursor[member]`; `pred` holds its branch predicate bits.
// With u == nullptr the pass is a plain gate pass and predicates are ignored.
struct TrajCtx {
    const double* u = nullptr;
    int64_t ustride = 0;
    const int64_t* cursor = nullptr;
    const uint64_t* pred = nullptr;
};

// Threads that compute on a tile (the pipelined kernel adds a producer warp beyond them).
constexpr int kCompute = 256;

// Barrier over the 256 compute threads only (named barrier 1): the pipelined kernel's producer
// warp never joins it. In the 256-thread kernel it spans the whole CTA.
__device__ __forceinline__ void cbar() { asm volatile("bar.sync 1, 256;" ::: "memory"); }

// The same barrier, returning whether any compute thread passed true.
__device__ __forceinline__ bool cbar_or(bool v) {
    uint32_t out;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.u32 p, %1, 0;\n\t"
        "bar.red.or.pred q, 1, 256, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}"
        : "=r"(out)
        : "r"((uint32_t)v)
        : "memory");
    return out != 0;
}

// Deposit the bits of x into the register positions listed in pos[0..n) (ascending).
__device__ __forceinline__ uint64_t deposit(uint64_t x, const int* pos, int n) {
    uint64_t out = 0;
    for (int j = 0; j < n; ++j) out |= ((x >> j) & 1ull) << pos[j];
    return out;
}

// Insert a zero bit at position b.
__device__ __forceinline__ uint32_t ins0(uint32_t g, int b) {
    const uint32_t low = g & ((1u << b) - 1);
    return ((g >> b) << (b + 1)) | low;
}

template <typename T>
__device__ __forceinline__ T ldm(const T* m, int i) {
    return m[i];
}

// 1-bit dense: the common case (fused one-qubit gates; one-qubit density superoperators use 2).
template <typename T>
__device__ __forceinline__ void dense1(T* t, int tbits, int b, const T* m) {
    const T m00 = m[0], m01 = m[1], m10 = m[2], m11 = m[3];
    const int groups = 1 << (tbits - 1);
    for (int g = threadIdx.x; g < groups; g += kCompute) {
        const uint32_t i0 = ins0((uint32_t)g, b), i1 = i0 | (1u << b);
        const T a0 = t[i0], a1 = t[i1];
        t[i0] = cfma(m01, a1, cmul(m00, a0));
        t[i1] = cfma(m11, a1, cmul(m10, a0));
    }
}

// 2-bit dense on (hi_bit = matrix MSB b0, b1); lo/hi are the sorted positions.
template <typename T>
__device__ __forceinline__ void dense2(T* t, int tbits, int b0, int b1, const T* m) {
    const int lo = min(b0, b1), hi = max(b0, b1);
    const uint32_t o1 = 1u << b1, o2 = 1u << b0;
    const int groups = 1 << (tbits - 2);
    for (int g = threadIdx.x; g < groups; g += kCompute) {
        const uint32_t base = ins0(ins0((uint32_t)g, lo), hi);
        const T v0 = t[base], v1 = t[base | o1], v2 = t[base | o2], v3 = t[base | o1 | o2];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            T acc = cmul(ldm(m, 4 * r), v0);
            acc = cfma(ldm(m, 4 * r + 1), v1, acc);
            acc = cfma(ldm(m, 4 * r + 2), v2, acc);
            acc = cfma(ldm(m, 4 * r + 3), v3, acc);
            const uint32_t at = base | ((r & 1) ? o1 : 0u) | ((r & 2) ? o2 : 0u);
            t[at] = acc;
        }
    }
}

template <typename T>
__device__ __forceinline__ T pick4(const T& v0, const T& v1, const T& v2, const T& v3, int s) {
    const T a = (s & 1) ? v1 : v0;
    const T b = (s & 1) ? v3 : v2;
    return (s & 2) ? b : a;
}

// permutations with phases on 1 or 2 bits (x, cx, swap and their phased forms)
template <typename T>
__device__ __forceinline__ void perm1(T* t, int tbits, int b, const T* m) {
    const T p0 = m[0], p1 = m[1];
    const int s0 = (int)re_of(m[2]);
    const int groups = 1 << (tbits - 1);
    for (int g = threadIdx.x; g < groups; g += kCompute) {
        const uint32_t i0 = ins0((uint32_t)g, b), i1 = i0 | (1u << b);
        const T a0 = t[i0], a1 = t[i1];
        t[i0] = cmul(p0, s0 ? a1 : a0);
        t[i1] = cmul(p1, s0 ? a0 : a1);
    }
}

template <typename T>
__device__ __forceinline__ void perm2(T* t, int tbits, int b0, int b1, const T* m) {
    const int lo = min(b0, b1), hi = max(b0, b1);
    const uint32_t o1 = 1u << b1, o2 = 1u << b0;
    const T p0 = m[0], p1 = m[1], p2 = m[2], p3 = m[3];
    const int s0 = (int)re_of(m[4]), s1 = (int)re_of(m[5]), s2 = (int)re_of(m[6]), s3 = (int)re_of(m[7]);
    const int groups = 1 << (tbits - 2);
    for (int g = threadIdx.x; g < groups; g += kCompute) {
        const uint32_t base = ins0(ins0((uint32_t)g, lo), hi);
        const T v0 = t[base], v1 = t[base | o1], v2 = t[base | o2], v3 = t[base | o1 | o2];
        t[base] = cmul(p0, pick4(v0, v1, v2, v3, s0));
        t[base | o1] = cmul(p1, pick4(v0, v1, v2, v3, s1));
        t[base | o2] = cmul(p2, pick4(v0, v1, v2, v3, s2));
        t[base | o1 | o2] = cmul(p3, pick4(v0, v1, v2, v3, s3));
    }
}

// Wide operators (3 to 5 bits): rare (Toffoli-class gates, two-qubit Kraus superoperators), kept
// out of line so their register needs don't shape the common path.
template <typename T>
__device__ __noinline__ void wide_op(T* t, int tbits, int kind, int k, const int* lb, const int* sorted,
                                     const T* m) {
    const int D = 1 << k;
    uint32_t offs[32];
    T v[32];
    for (int j = 0; j < D; ++j) {
        uint32_t o = 0;
        for (int i = 0; i < k; ++i) o |= (uint32_t)((j >> (k - 1 - i)) & 1) << lb[i];
        offs[j] = o;
    }
    const int groups = 1 << (tbits - k);
    for (int g = threadIdx.x; g < groups; g += kCompute) {
        uint32_t base = (uint32_t)g;
        for (int i = 0; i < k; ++i) base = ins0(base, sorted[i]);
        for (int j = 0; j < D; ++j) v[j] = t[base | offs[j]];
        if (kind == LSG_OP_MATRIX) {
            for (int r = 0; r < D; ++r) {
                T acc{};
                for (int c = 0; c < D; ++c) acc = cfma(m[r * D + c], v[c], acc);
                t[base | offs[r]] = acc;
            }
        } else {
            for (int r = 0; r < D; ++r) t[base | offs[r]] = cmul(m[r], v[(int)re_of(m[D + r])]);
        }
    }
}

template <typename T>
__device__ __forceinline__ void op_diag(T* tile, int tbits, int k, const int* lb, const T* m) {
    const int n = 1 << tbits;
    for (int i = threadIdx.x; i < n; i += kCompute) {
        int j = 0;
        for (int b = 0; b < k; ++b) j = (j << 1) | ((i >> lb[b]) & 1);
        tile[i] = cmul(m[j], tile[i]);
    }
}

template <typename T>
__device__ __forceinline__ void op_scale(T* tile, int tbits, const T* m) {
    const int n = 1 << tbits;
    const T f = m[0];
    for (int i = threadIdx.x; i < n; i += kCompute) tile[i] = cmul(f, tile[i]);
}

// (1-p) rho + (p/d) I (x) Tr_t(rho) on kq row bits then kq column bits (kq = 1 or 2).
template <typename T, int KQ>
__device__ __forceinline__ void op_depol(T* t, int tbits, const int* lb, const int* sorted, const T* m) {
    using R = typename Elem<T>::R;
    if constexpr (Elem<T>::complex) {
    constexpr int KB = 2 * KQ;
    constexpr int D = 1 << KB;
    constexpr int d = 1 << KQ;
    int l[KB], srt[KB];
#pragma unroll
    for (int i = 0; i < KB; ++i) {
        l[i] = lb[i];
        srt[i] = sorted[i];
    }
    const R p = m[0].re;
    const R keep = R(1) - p;
    const R share = p / R(d);
    const int groups = 1 << (tbits - KB);
    for (int g = threadIdx.x; g < groups; g += kCompute) {
        uint32_t base = (uint32_t)g;
#pragma unroll
        for (int i = 0; i < KB; ++i) base = ins0(base, srt[i]);
        T tr;
#pragma unroll
        for (int s = 0; s < d; ++s) {
            const int j = (s << KQ) | s;
            uint32_t o = 0;
#pragma unroll
            for (int i = 0; i < KB; ++i) o |= (uint32_t)((j >> (KB - 1 - i)) & 1) << l[i];
            const T v = t[base | o];
            tr.re += v.re;
            tr.im += v.im;
        }
#pragma unroll
        for (int j = 0; j < D; ++j) {
            uint32_t o = 0;
#pragma unroll
            for (int i = 0; i < KB; ++i) o |= (uint32_t)((j >> (KB - 1 - i)) & 1) << l[i];
            const T v = t[base | o];
            T out(v.re * keep, v.im * keep);
            if ((j >> KQ) == (j & (d - 1))) {
                out.re += share * tr.re;
                out.im += share * tr.im;
            }
            t[base | o] = out;
        }
    }
    }
}

// A state-independent noise channel in a trajectory: the member picks branch i, the first with
// u < cum[i] (cum = running sums of the branch probabilities, as engines.py:163-171 accumulates
// them), and applies that branch's unitary unless it is the identity. Data: `count` entries
// (re = cumulative probability, im = 1 for an identity branch), then `count` dense 2^k matrices.
template <typename T>
__device__ __forceinline__ void op_mixture(T* t, int tbits, const TileOp& op, const T* m, double u) {
    using R = typename Elem<T>::R;
    if constexpr (Elem<T>::complex) {
    const int nb = op.count;
    int pick = -1;
    for (int i = 0; i < nb; ++i) {
        if (u < (double)m[i].re) {
            pick = i;
            break;
        }
    }
    if (pick < 0 || m[pick].im != R(0)) return;  // nothing drawn, or the identity branch
    const int d = 1 << op.k;
    const T* mat = m + nb + (int64_t)pick * d * d;
    if (op.k == 1) dense1<T>(t, tbits, op.lb[0], mat);
    else if (op.k == 2) dense2<T>(t, tbits, op.lb[0], op.lb[1], mat);
    else wide_op<T>(t, tbits, LSG_OP_MATRIX, op.k, op.lb, op.sorted, mat);
    }
}


// ------------------------------------------------------------------ register blocks
//
// v[e] holds the amplitude at group offset e of a block of U bits; bit (U-1-P) of e is block
// position P. Every function below is fully unrolled over e, so v stays in registers.

// N operator entries into registers with 16-byte loads (the host places register-block operator
// data on 16-byte boundaries).
__device__ __forceinline__ void ld16(const float* p, float* o) {
    const float4 w = __ldg(reinterpret_cast<const float4*>(p));
    o[0] = w.x, o[1] = w.y, o[2] = w.z, o[3] = w.w;
}
__device__ __forceinline__ void ld16(const double* p, double* o) {
    const double2 w = __ldg(reinterpret_cast<const double2*>(p));
    o[0] = w.x, o[1] = w.y;
}
__device__ __forceinline__ void ld16(const DF* p, DF* o) {
    const float4 w = __ldg(reinterpret_cast<const float4*>(p));
    o[0] = DF(w.x, w.y), o[1] = DF(w.z, w.w);
}
__device__ __forceinline__ void ld16(const Cx<float>* p, Cx<float>* o) {
    const float4 w = __ldg(reinterpret_cast<const float4*>(p));
    o[0] = Cx<float>(w.x, w.y), o[1] = Cx<float>(w.z, w.w);
}
__device__ __forceinline__ void ld16(const Cx<double>* p, Cx<double>* o) {
    const double2 w = __ldg(reinterpret_cast<const double2*>(p));
    o[0] = Cx<double>(w.x, w.y);
}

template <typename T, int N>
__device__ __forceinline__ void ldv(const T* __restrict__ m, T* out) {
    static_assert((N * sizeof(T)) % 16 == 0, "whole 16-byte words");
    constexpr int per = 16 / sizeof(T);
#pragma unroll
    for (int i = 0; i < N / per; ++i) ld16(m + i * per, out + i * per);
}

template <typename T, int U, int P>
__device__ __forceinline__ void rb_dense1(T* v, const T* m) {
    constexpr int B = 1 << (U - 1 - P);
    T mm[4];
    ldv<T, 4>(m, mm);
    const T m00 = mm[0], m01 = mm[1], m10 = mm[2], m11 = mm[3];
#pragma unroll
    for (int e = 0; e < (1 << U); ++e) {
        if (e & B) continue;
        const T a0 = v[e], a1 = v[e | B];
        v[e] = cfma(m01, a1, cmul(m00, a0));
        v[e | B] = cfma(m11, a1, cmul(m10, a0));
    }
}

template <typename T, int U, int P0, int P1>
__device__ __forceinline__ void rb_dense2(T* v, const T* m) {
    constexpr int B0 = 1 << (U - 1 - P0), B1 = 1 << (U - 1 - P1);
    T mm[16];
    ldv<T, 16>(m, mm);
#pragma unroll
    for (int e = 0; e < (1 << U); ++e) {
        if (e & (B0 | B1)) continue;
        const T a0 = v[e], a1 = v[e | B1], a2 = v[e | B0], a3 = v[e | B0 | B1];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            T acc = cmul(mm[4 * r], a0);
            acc = cfma(mm[4 * r + 1], a1, acc);
            acc = cfma(mm[4 * r + 2], a2, acc);
            acc = cfma(mm[4 * r + 3], a3, acc);
            v[e | ((r & 2) ? B0 : 0) | ((r & 1) ? B1 : 0)] = acc;
        }
    }
}

// A real 4x4 transfer matrix with first row (1,0,0,0) (trace preserving): output 0 keeps its
// input, rows 1-3 are computed. 12 multiply-adds per 4 elements instead of 16. Z (specialized
// passes) marks coefficients that are exactly zero for every member, bit 4 * (r - 1) + c for
// row r, column c: their terms are left out. A zero term adds an exact zero to the row's sum, so
// leaving it out gives the same values (a noisy one-qubit gate's X and Y rows have a zero first
// column: 10 multiply-adds per 4 elements).
template <typename T, int U, int P0, int P1, int Z = 0>
__device__ __forceinline__ void rb_tpd2(T* v, const T* m) {
    if constexpr (!Elem<T>::complex) {
        constexpr int B0 = 1 << (U - 1 - P0), B1 = 1 << (U - 1 - P1);
        T mm[12];
        ldv<T, 12>(m + 4, mm);
#pragma unroll
        for (int e = 0; e < (1 << U); ++e) {
            if (e & (B0 | B1)) continue;
            const T a[4] = {v[e], v[e | B1], v[e | B0], v[e | B0 | B1]};
#pragma unroll
            for (int r = 1; r < 4; ++r) {
                T acc{};
                if constexpr (IsDF<T>::value) {  // one renormalisation per row
                    acc = df_dot<4>(mm + 4 * r - 4, a, (unsigned)(Z >> (4 * (r - 1))) & 15u);
                } else {
                    bool first = true;
#pragma unroll
                    for (int c = 0; c < 4; ++c) {
                        if (Z & (1 << (4 * (r - 1) + c))) continue;
                        acc = first ? cmul(mm[4 * r - 4 + c], a[c]) : cfma(mm[4 * r - 4 + c], a[c], acc);
                        first = false;
                    }
                }
                v[e | ((r & 2) ? B0 : 0) | ((r & 1) ? B1 : 0)] = acc;
            }
        }
    }
}

template <typename T, int U, int P>
__device__ __forceinline__ void rb_perm1(T* v, const T* m) {
    constexpr int B = 1 << (U - 1 - P);
    const T p0 = m[0], p1 = m[1];
    const bool swap = re_of(m[2]) != 0;
#pragma unroll
    for (int e = 0; e < (1 << U); ++e) {
        if (e & B) continue;
        const T a0 = v[e], a1 = v[e | B];
        v[e] = cmul(p0, swap ? a1 : a0);
        v[e | B] = cmul(p1, swap ? a0 : a1);
    }
}

template <typename T, int U, int P0, int P1>
__device__ __forceinline__ void rb_perm2(T* v, const T* m) {
    constexpr int B0 = 1 << (U - 1 - P0), B1 = 1 << (U - 1 - P1);
    const T p0 = m[0], p1 = m[1], p2 = m[2], p3 = m[3];
    const int s0 = (int)re_of(m[4]), s1 = (int)re_of(m[5]), s2 = (int)re_of(m[6]), s3 = (int)re_of(m[7]);
#pragma unroll
    for (int e = 0; e < (1 << U); ++e) {
        if (e & (B0 | B1)) continue;
        const T a0 = v[e], a1 = v[e | B1], a2 = v[e | B0], a3 = v[e | B0 | B1];
        v[e] = cmul(p0, pick4(a0, a1, a2, a3, s0));
        v[e | B1] = cmul(p1, pick4(a0, a1, a2, a3, s1));
        v[e | B0] = cmul(p2, pick4(a0, a1, a2, a3, s2));
        v[e | B0 | B1] = cmul(p3, pick4(a0, a1, a2, a3, s3));
    }
}

// A whole register block fused on the host into one dense 2^U x 2^U complex matrix (row-major,
// rows and columns in block order): out[r] = sum_c m[r][c] v[c]. The host forms the product of
// the block's operators in FP64 and rounds it once to the register precision.
template <typename T, int U>
__device__ __forceinline__ void rb_denseb(T* v, const T* m) {
    constexpr int D = 1 << U;
    T out[D];
#pragma unroll
    for (int r = 0; r < D; ++r) {
        T row[4];  // the row in 4-entry pieces: few registers beside the group and the outputs
        ldv<T, 4>(m + r * D, row);
        T acc = cmul(row[0], v[0]);
#pragma unroll
        for (int c = 1; c < D; ++c) {
            if ((c & 3) == 0) ldv<T, 4>(m + r * D + c, row);
            acc = cfma(row[c & 3], v[c], acc);
        }
        out[r] = acc;
    }
#pragma unroll
    for (int e = 0; e < D; ++e) v[e] = out[e];
}

// The interpreter's form of rb_denseb: the group is in registers, each output row is stored to
// the tile as soon as it is formed (the group's elements belong to this thread alone).
template <typename T, int U>
__device__ __forceinline__ void rb_denseb_store(T* tile, uint32_t base, const uint32_t* off, const T* v, const T* m) {
    constexpr int D = 1 << U;
#pragma unroll
    for (int r = 0; r < D; ++r) {
        T row[4];
        ldv<T, 4>(m + r * D, row);
        T acc = cmul(row[0], v[0]);
#pragma unroll
        for (int c = 1; c < D; ++c) {
            if ((c & 3) == 0) ldv<T, 4>(m + r * D + c, row);
            acc = cfma(row[c & 3], v[c], acc);
        }
        tile[base | off[r]] = acc;
    }
}

// Unit-phase permutations are register renames: no arithmetic at all.
template <typename T, int U, int P>
__device__ __forceinline__ void rb_x(T* v) {
    constexpr int B = 1 << (U - 1 - P);
#pragma unroll
    for (int e = 0; e < (1 << U); ++e)
        if (!(e & B)) {
            const T t = v[e];
            v[e] = v[e | B];
            v[e | B] = t;
        }
}

// controlled X: control at position PC, target at PT
template <typename T, int U, int PC, int PT>
__device__ __forceinline__ void rb_cx(T* v) {
    constexpr int BC = 1 << (U - 1 - PC), BT = 1 << (U - 1 - PT);
#pragma unroll
    for (int e = 0; e < (1 << U); ++e)
        if ((e & BC) && !(e & BT)) {
            const T t = v[e];
            v[e] = v[e | BT];
            v[e | BT] = t;
        }
}

template <typename T, int U, int P0, int P1>
__device__ __forceinline__ void rb_swap(T* v) {
    constexpr int B0 = 1 << (U - 1 - P0), B1 = 1 << (U - 1 - P1);
#pragma unroll
    for (int e = 0; e < (1 << U); ++e)
        if ((e & B0) && !(e & B1)) {
            const T t = v[e];
            v[e] = v[(e & ~B0) | B1];
            v[(e & ~B0) | B1] = t;
        }
}

// (1-p) rho + (p/2) I Tr on one row bit (position PR) and its column bit (PC)
template <typename T, int U, int PR, int PC>
__device__ __forceinline__ void rb_depol1(T* v, const T* m) {
    using R = typename Elem<T>::R;
    if constexpr (Elem<T>::complex) {
    constexpr int BR = 1 << (U - 1 - PR), BC = 1 << (U - 1 - PC);
    const R p = m[0].re, keep = R(1) - p, share = p / R(2);
#pragma unroll
    for (int e = 0; e < (1 << U); ++e) {
        if (e & (BR | BC)) continue;
        const T d0 = v[e], d1 = v[e | BR | BC];
        const T tr(d0.re + d1.re, d0.im + d1.im);
        v[e] = T(d0.re * keep + share * tr.re, d0.im * keep + share * tr.im);
        v[e | BR | BC] = T(d1.re * keep + share * tr.re, d1.im * keep + share * tr.im);
        const T o1 = v[e | BC], o2 = v[e | BR];
        v[e | BC] = T(o1.re * keep, o1.im * keep);
        v[e | BR] = T(o2.re * keep, o2.im * keep);
    }
    }
}

// two-qubit form on positions (row a, row b, col a, col b) = (0, 1, 2, 3) of a 4-bit block
template <typename T>
__device__ __forceinline__ void rb_depol2(T* v, const T* m) {
    using R = typename Elem<T>::R;
    if constexpr (Elem<T>::complex) {
    const R p = m[0].re, keep = R(1) - p, share = p / R(4);
    T tr;
#pragma unroll
    for (int t = 0; t < 4; ++t) {
        tr.re += v[(t << 2) | t].re;
        tr.im += v[(t << 2) | t].im;
    }
#pragma unroll
    for (int e = 0; e < 16; ++e) {
        T o(v[e].re * keep, v[e].im * keep);
        if ((e >> 2) == (e & 3)) {
            o.re += share * tr.re;
            o.im += share * tr.im;
        }
        v[e] = o;
    }
    }
}

// a diagonal whose 2^U entries the host laid out in block order (no index arithmetic)
template <typename T, int U>
__device__ __forceinline__ void rb_diagb(T* v, const T* m) {
    if constexpr (((1 << U) * sizeof(T)) % 16 == 0) {
        T mm[1 << U];
        ldv<T, (1 << U)>(m, mm);
#pragma unroll
        for (int e = 0; e < (1 << U); ++e) v[e] = cmul(mm[e], v[e]);
    } else {
#pragma unroll
        for (int e = 0; e < (1 << U); ++e) v[e] = cmul(m[e], v[e]);
    }
}

template <typename T, int U>
__device__ __forceinline__ void rb_scale(T* v, const T* m) {
    const T f = m[0];
#pragma unroll
    for (int e = 0; e < (1 << U); ++e) v[e] = cmul(f, v[e]);
}

// ------------------------------------------------------------------ packed group pairs (real32)
//
// A specialized pass whose block leaves tile bit 0 free handles two groups per thread (tile bit 0
// clear and set). For real32 registers the pair's two values of element e can live in one 64-bit
// register pair and every operator runs on both with one packed FP32 instruction (mul.rn.f32x2,
// fma.rn.f32x2, sm_100 and later): lane 0 is the group with tile bit 0 clear. Each lane is
// rounded exactly as the scalar mul / fma of the unpacked form, in the same order, so results
// are identical bit for bit; the coefficient is broadcast to both lanes.
struct F2 {
    unsigned long long r;
};
__device__ __forceinline__ F2 f2_bcast(float c) {
    F2 o;
    asm("mov.b64 %0, {%1, %1};" : "=l"(o.r) : "f"(c));
    return o;
}
__device__ __forceinline__ F2 f2_mul(float c, F2 a) {
    F2 o;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(o.r) : "l"(f2_bcast(c).r), "l"(a.r));
    return o;
}
__device__ __forceinline__ F2 f2_fma(float c, F2 a, F2 acc) {
    F2 o;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(o.r) : "l"(f2_bcast(c).r), "l"(a.r), "l"(acc.r));
    return o;
}
// the pair at p (8-byte aligned): p[0] to lane 0, p[1] to lane 1
__device__ __forceinline__ F2 ld_f2(const float* p) {
    F2 o;
    o.r = *reinterpret_cast<const unsigned long long*>(p);
    return o;
}
__device__ __forceinline__ void st_f2(float* p, F2 v) { *reinterpret_cast<unsigned long long*>(p) = v.r; }

template <int U, int P>
__device__ __forceinline__ void rp_dense1(F2* v, const float* m) {
    constexpr int B = 1 << (U - 1 - P);
    float mm[4];
    ldv<float, 4>(m, mm);
#pragma unroll
    for (int e = 0; e < (1 << U); ++e) {
        if (e & B) continue;
        const F2 a0 = v[e], a1 = v[e | B];
        v[e] = f2_fma(mm[1], a1, f2_mul(mm[0], a0));
        v[e | B] = f2_fma(mm[3], a1, f2_mul(mm[2], a0));
    }
}

template <int U, int P0, int P1>
__device__ __forceinline__ void rp_dense2(F2* v, const float* m) {
    constexpr int B0 = 1 << (U - 1 - P0), B1 = 1 << (U - 1 - P1);
    float mm[16];
    ldv<float, 16>(m, mm);
#pragma unroll
    for (int e = 0; e < (1 << U); ++e) {
        if (e & (B0 | B1)) continue;
        const F2 a0 = v[e], a1 = v[e | B1], a2 = v[e | B0], a3 = v[e | B0 | B1];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            F2 acc = f2_mul(mm[4 * r], a0);
            acc = f2_fma(mm[4 * r + 1], a1, acc);
            acc = f2_fma(mm[4 * r + 2], a2, acc);
            acc = f2_fma(mm[4 * r + 3], a3, acc);
            v[e | ((r & 2) ? B0 : 0) | ((r & 1) ? B1 : 0)] = acc;
        }
    }
}

template <int U, int P0, int P1, int Z = 0>
__device__ __forceinline__ void rp_tpd2(F2* v, const float* m) {
    constexpr int B0 = 1 << (U - 1 - P0), B1 = 1 << (U - 1 - P1);
    float mm[12];
    ldv<float, 12>(m + 4, mm);
#pragma unroll
    for (int e = 0; e < (1 << U); ++e) {
        if (e & (B0 | B1)) continue;
        const F2 a[4] = {v[e], v[e | B1], v[e | B0], v[e | B0 | B1]};
#pragma unroll
        for (int r = 1; r < 4; ++r) {
            F2 acc = f2_bcast(0.0f);
            bool first = true;
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                if (Z & (1 << (4 * (r - 1) + c))) continue;
                acc = first ? f2_mul(mm[4 * r - 4 + c], a[c]) : f2_fma(mm[4 * r - 4 + c], a[c], acc);
                first = false;
            }
            v[e | ((r & 2) ? B0 : 0) | ((r & 1) ? B1 : 0)] = acc;
        }
    }
}

template <int U, int P>
__device__ __forceinline__ void rp_perm1(F2* v, const float* m) {
    constexpr int B = 1 << (U - 1 - P);
    const float p0 = m[0], p1 = m[1];
    const bool swap = m[2] != 0.0f;
#pragma unroll
    for (int e = 0; e < (1 << U); ++e) {
        if (e & B) continue;
        const F2 a0 = v[e], a1 = v[e | B];
        v[e] = f2_mul(p0, swap ? a1 : a0);
        v[e | B] = f2_mul(p1, swap ? a0 : a1);
    }
}

template <int U, int P0, int P1>
__device__ __forceinline__ void rp_perm2(F2* v, const float* m) {
    constexpr int B0 = 1 << (U - 1 - P0), B1 = 1 << (U - 1 - P1);
    const float p0 = m[0], p1 = m[1], p2 = m[2], p3 = m[3];
    const int s0 = (int)m[4], s1 = (int)m[5], s2 = (int)m[6], s3 = (int)m[7];
#pragma unroll
    for (int e = 0; e < (1 << U); ++e) {
        if (e & (B0 | B1)) continue;
        const F2 a0 = v[e], a1 = v[e | B1], a2 = v[e | B0], a3 = v[e | B0 | B1];
        v[e] = f2_mul(p0, pick4(a0, a1, a2, a3, s0));
        v[e | B1] = f2_mul(p1, pick4(a0, a1, a2, a3, s1));
        v[e | B0] = f2_mul(p2, pick4(a0, a1, a2, a3, s2));
        v[e | B0 | B1] = f2_mul(p3, pick4(a0, a1, a2, a3, s3));
    }
}

template <int U>
__device__ __forceinline__ void rp_diagb(F2* v, const float* m) {
    if constexpr (((1 << U) * 4) % 16 == 0) {
        float mm[1 << U];
        ldv<float, (1 << U)>(m, mm);
#pragma unroll
        for (int e = 0; e < (1 << U); ++e) v[e] = f2_mul(mm[e], v[e]);
    } else {
#pragma unroll
        for (int e = 0; e < (1 << U); ++e) v[e] = f2_mul(m[e], v[e]);
    }
}

template <int U>
__device__ __forceinline__ void rp_scale(F2* v, const float* m) {
    const float f = m[0];
#pragma unroll
    for (int e = 0; e < (1 << U); ++e) v[e] = f2_mul(f, v[e]);
}

// the branch matrix a member's uniform picks from a mixture channel, or nullptr for identity
template <typename T>
__device__ __forceinline__ const T* mixture_pick(const TileOp& op, const T* m, double u) {
    using R = typename Elem<T>::R;
    if constexpr (Elem<T>::complex) {
    const int nb = op.count;
    int pick = -1;
    for (int i = 0; i < nb; ++i)
        if (u < (double)m[i].re) {
            pick = i;
            break;
        }
    if (pick < 0 || m[pick].im != R(0)) return nullptr;
    const int d = 1 << op.k;
    return m + nb + (int64_t)pick * d * d;
    }
    return nullptr;
}

// Case lists of rb_apply: a register-block code names the operator's positions P in the block.
#define LSG_P1(X, BASE)                                                                  \
    case BASE + 0: if (U > 0) X<T, U, (0 < U ? 0 : 0)>(v, m); break; \
    case BASE + 1: if (U > 1) X<T, U, (1 < U ? 1 : 0)>(v, m); break; \
    case BASE + 2: if (U > 2) X<T, U, (2 < U ? 2 : 0)>(v, m); break; \
    case BASE + 3: if (U > 3) X<T, U, (3 < U ? 3 : 0)>(v, m); break;

#define LSG_P2ONE(X, BASE, A, B)                                                                        \
    case BASE + 4 * A + B:                                                                              \
        if (U > A && U > B) X<T, U, (A < U ? A : 0), (B < U ? B : 0)>(v, m); \
        break;

#define LSG_R1(X, BASE)                                                               \
    case BASE + 0: if (U > 0) X<T, U, (0 < U ? 0 : 0)>(v); break; \
    case BASE + 1: if (U > 1) X<T, U, (1 < U ? 1 : 0)>(v); break; \
    case BASE + 2: if (U > 2) X<T, U, (2 < U ? 2 : 0)>(v); break; \
    case BASE + 3: if (U > 3) X<T, U, (3 < U ? 3 : 0)>(v); break;

#define LSG_R2ONE(X, BASE, A, B)                                                                     \
    case BASE + 4 * A + B:                                                                           \
        if (U > A && U > B) X<T, U, (A < U ? A : 0), (B < U ? B : 0)>(v); \
        break;

// two positions never coincide: those four codes are empty cases that keep the switch dense
#define LSG_SAME(BASE) \
    case BASE + 0: case BASE + 5: case BASE + 10: case BASE + 15: break;

#define LSG_R2(X, BASE)                                                                                  \
    LSG_R2ONE(X, BASE, 0, 1) LSG_R2ONE(X, BASE, 0, 2) LSG_R2ONE(X, BASE, 0, 3) LSG_R2ONE(X, BASE, 1, 0) \
    LSG_R2ONE(X, BASE, 1, 2) LSG_R2ONE(X, BASE, 1, 3) LSG_R2ONE(X, BASE, 2, 0) LSG_R2ONE(X, BASE, 2, 1) \
    LSG_R2ONE(X, BASE, 2, 3) LSG_R2ONE(X, BASE, 3, 0) LSG_R2ONE(X, BASE, 3, 1) LSG_R2ONE(X, BASE, 3, 2) \
    LSG_SAME(BASE)

#define LSG_P2(X, BASE)                                                                                  \
    LSG_P2ONE(X, BASE, 0, 1) LSG_P2ONE(X, BASE, 0, 2) LSG_P2ONE(X, BASE, 0, 3) LSG_P2ONE(X, BASE, 1, 0) \
    LSG_P2ONE(X, BASE, 1, 2) LSG_P2ONE(X, BASE, 1, 3) LSG_P2ONE(X, BASE, 2, 0) LSG_P2ONE(X, BASE, 2, 1) \
    LSG_P2ONE(X, BASE, 2, 3) LSG_P2ONE(X, BASE, 3, 0) LSG_P2ONE(X, BASE, 3, 1) LSG_P2ONE(X, BASE, 3, 2) \
    LSG_SAME(BASE)

template <typename T, int U>
__device__ __forceinline__ void rb_apply(T* v, int code, const T* m) {
    switch (code) {
        LSG_P1(rb_dense1, kT_DENSE1)
        LSG_P2(rb_dense2, kT_DENSE2)
        LSG_P2(rb_tpd2, kT_TPD2)
        LSG_P1(rb_perm1, kT_PERM1)
        LSG_P2(rb_perm2, kT_PERM2)
        LSG_P2(rb_depol1, kT_DEPOL1)
        case kT_DEPOL2:
            if constexpr (U == 4) rb_depol2<T>(v, m);
            break;
        LSG_R1(rb_x, kT_X1)
        LSG_R2(rb_cx, kT_CX)
        LSG_R2(rb_swap, kT_SWAP)
        case kT_DIAGB: rb_diagb<T, U>(v, m); break;
        case kT_SCALE: rb_scale<T, U>(v, m); break;

        default: break;
    }
}

// A group's 2^U elements between shared memory and registers. With vec = 2 or 4 the group's last
// positions are tile bits (1,) 0: runs of consecutive elements, moved with 8- or 16-byte accesses
// where the element size allows (the run's address is then aligned: base and off[] have those bits
// clear).
template <typename T, int U>
__device__ __forceinline__ void load_group(const T* tile, uint32_t base, const uint32_t* off, int vec, T* v) {
    if constexpr (sizeof(T) == 4 && U >= 2) {
        if (vec == 4) {
#pragma unroll
            for (int e = 0; e < (1 << U); e += 4) {
                const float4 w = *reinterpret_cast<const float4*>(tile + (base | off[e]));
                v[e] = w.x, v[e + 1] = w.y, v[e + 2] = w.z, v[e + 3] = w.w;
            }
            return;
        }
    }
    if constexpr (sizeof(T) == 8 && U >= 1) {
        if (vec >= 2) {
#pragma unroll
            for (int e = 0; e < (1 << U); e += 2) {
                const uint4 w = *reinterpret_cast<const uint4*>(tile + (base | off[e]));
                memcpy(&v[e], &w.x, 8);
                memcpy(&v[e + 1], &w.z, 8);
            }
            return;
        }
    }
    if constexpr (sizeof(T) == 4 && U >= 1) {
        if (vec == 2) {
#pragma unroll
            for (int e = 0; e < (1 << U); e += 2) {
                const float2 w = *reinterpret_cast<const float2*>(tile + (base | off[e]));
                v[e] = w.x, v[e + 1] = w.y;
            }
            return;
        }
    }
#pragma unroll
    for (int e = 0; e < (1 << U); ++e) v[e] = tile[base | off[e]];
}

template <typename T, int U>
__device__ __forceinline__ void store_group(T* tile, uint32_t base, const uint32_t* off, int vec, const T* v) {
    if constexpr (sizeof(T) == 4 && U >= 2) {
        if (vec == 4) {
#pragma unroll
            for (int e = 0; e < (1 << U); e += 4)
                *reinterpret_cast<float4*>(tile + (base | off[e])) = make_float4(v[e], v[e + 1], v[e + 2], v[e + 3]);
            return;
        }
    }
    if constexpr (sizeof(T) == 8 && U >= 1) {
        if (vec >= 2) {
#pragma unroll
            for (int e = 0; e < (1 << U); e += 2) {
                uint4 w;
                memcpy(&w.x, &v[e], 8);
                memcpy(&w.z, &v[e + 1], 8);
                *reinterpret_cast<uint4*>(tile + (base | off[e])) = w;
            }
            return;
        }
    }
    if constexpr (sizeof(T) == 4 && U >= 1) {
        if (vec == 2) {
#pragma unroll
            for (int e = 0; e < (1 << U); e += 2)
                *reinterpret_cast<float2*>(tile + (base | off[e])) = make_float2(v[e], v[e + 1]);
            return;
        }
    }
#pragma unroll
    for (int e = 0; e < (1 << U); ++e) tile[base | off[e]] = v[e];
}

// A register-block operator resolved for the tile's member: its code and data pointer (built
// once per tile in shared memory, so the inner loop reads one 16-byte record per operator).
struct OpRec {
    int code, pad;
    const void* m;
};

// One register block over the whole tile: each thread takes groups of 2^U elements (the block's
// U register bits), reads them, applies the block's operators (records resolved for the tile's
// member) in registers and writes them back.
template <typename T, int U>
__device__ void run_block(T* tile, int tbits, const BlockDesc& blk, const OpRec* __restrict__ recs) {
    // element e of a group sits at base | off[e]: the block's bits of e deposited at its tile bits
    uint32_t off[1 << U];
#pragma unroll
    for (int e = 0; e < (1 << U); ++e) {
        uint32_t a = 0;
#pragma unroll
        for (int i = 0; i < U; ++i)
            if ((e >> (U - 1 - i)) & 1) a |= 1u << blk.bits[i];
        off[e] = a;
    }
    const int groups = 1 << (tbits - U);
    const bool dense = blk.nops == 1 && recs[blk.first].code == kT_DENSEB;
    for (int g = threadIdx.x; g < groups; g += kCompute) {
        uint32_t base = 0;
#pragma unroll
        for (int i = 0; i <= U; ++i) base |= ((uint32_t)g << i) & blk.dep[i];
        T v[1 << U];
        load_group<T, U>(tile, base, off, blk.vec, v);
        if constexpr (Elem<T>::complex) {
            if (dense) {  // a fused block: each output row straight back to its place in the tile
                rb_denseb_store<T, U>(tile, base, off, v, static_cast<const T*>(recs[blk.first].m));
                continue;
            }
        }
        for (int o = 0; o < blk.nops; ++o) {
            const OpRec r = recs[blk.first + o];
            rb_apply<T, U>(v, r.code, static_cast<const T*>(r.m));
        }
        store_group<T, U>(tile, base, off, blk.vec, v);
    }
}

template <typename T>
__device__ void run_ops(T* tile, int tbits, const TileOp* __restrict__ ops, int nops,
                        const T* __restrict__ data, int64_t member, const TrajCtx& ctx) {
    const uint64_t pred = ctx.u ? ctx.pred[member] : ~0ull;
    const int64_t cur = ctx.u ? ctx.cursor[member] : 0;
    for (int o = 0; o < nops; ++o) {
        const TileOp& op = ops[o];  // staged in shared memory
        const int kind = op.kind, k = op.k;
        const T* m = data + op.data + member * op.stride;
        if (!((pred >> op.pred) & 1)) continue;  // a branch this member did not take (CTA-uniform)
        cbar();
        if (kind == kOpMixture) {
            op_mixture<T>(tile, tbits, op, m, ctx.u[member * ctx.ustride + cur + op.draw]);
        } else if (kind == LSG_OP_MATRIX && k == 1) {
            dense1<T>(tile, tbits, op.lb[0], m);
        } else if (kind == LSG_OP_MATRIX && k == 2) {
            dense2<T>(tile, tbits, op.lb[0], op.lb[1], m);
        } else if (kind == LSG_OP_PERM && k == 1) {
            perm1<T>(tile, tbits, op.lb[0], m);
        } else if (kind == LSG_OP_PERM && k == 2) {
            perm2<T>(tile, tbits, op.lb[0], op.lb[1], m);
        } else if (kind == LSG_OP_DIAG) {
            op_diag<T>(tile, tbits, k, op.lb, m);
        } else if (kind == LSG_OP_DEPOL) {
            if (k == 2) op_depol<T, 1>(tile, tbits, op.lb, op.sorted, m);
            else op_depol<T, 2>(tile, tbits, op.lb, op.sorted, m);
        } else if (kind == LSG_OP_SCALE) {
            op_scale<T>(tile, tbits, m);
        } else {
            wide_op<T>(tile, tbits, kind, k, op.lb, op.sorted, m);
        }
    }
    cbar();
}

// All blocks of a pass on one tile (the 256 compute threads).
template <typename T>
__device__ __forceinline__ void compute_tile(T* tile, int K, const PassDesc& pd, const BlockDesc* sblk,
                                             const TileOp* sops, OpRec* recs, const T* __restrict__ data,
                                             int64_t member, const TrajCtx& ctx) {
    const bool plain = ctx.u == nullptr;
    const uint64_t pred = plain ? ~0ull : ctx.pred[member];
    const int64_t cur = plain ? 0 : ctx.cursor[member];
    // this tile's member: resolve every operator once — its data pointer and, in a trajectory
    // pass, its predicate (an untaken branch gets code -1: no operation) and its mixture branch
    // (drawn from the member's uniform; the identity branch is skipped like an untaken one)
    for (int o = threadIdx.x; o < pd.nops; o += kCompute) {
        const TileOp& op = sops[o];
        int code = op.tmpl;
        const T* m = data + op.data + member * op.stride;
        if (!plain) {
            if (!((pred >> op.pred) & 1)) {
                code = -1;
            } else if (op.kind == kOpMixture) {
                m = mixture_pick<T>(op, m, ctx.u[member * ctx.ustride + cur + op.draw]);
                code = m ? (op.k == 1 ? kT_DENSE1 : kT_DENSE2) + (code - (op.k == 1 ? kT_MIX1 : kT_MIX2)) : -1;
            }
        }
        recs[o] = OpRec{code, 0, m};
    }
    for (int bi = 0; bi < pd.nblocks; ++bi) {
        const BlockDesc& blk = sblk[bi];
        cbar();
        if (blk.generic) {
            run_ops<T>(tile, K, sops + blk.first, blk.nops, data, member, ctx);
            continue;
        }
#define LSG_RUN(UU) run_block<T, UU>(tile, K, blk, recs);
        switch (blk.u) {
            case 1: LSG_RUN(1) break;
            case 2: LSG_RUN(2) break;
            case 3: LSG_RUN(3) break;
            default:
                if constexpr (sizeof(T) <= 8) {
                    LSG_RUN(4)
                }
                break;
        }
#undef LSG_RUN
    }
    cbar();
}

template <typename T>
__device__ __forceinline__ void stage_pass(const PassDesc* __restrict__ pass_g, const TileOp* __restrict__ ops,
                                           const BlockDesc* __restrict__ blocks, TileOp* sops, BlockDesc* sblk) {
    const int nops = pass_g->nops;
    const int* src = reinterpret_cast<const int*>(ops + pass_g->first_op);
    int* dst = reinterpret_cast<int*>(sops);
    const int words = nops * (int)(sizeof(TileOp) / sizeof(int));
    for (int i = threadIdx.x; i < words; i += blockDim.x) dst[i] = src[i];
    const int* bsrc = reinterpret_cast<const int*>(blocks + pass_g->first_block);
    int* bdst = reinterpret_cast<int*>(sblk);
    const int bwords = pass_g->nblocks * (int)(sizeof(BlockDesc) / sizeof(int));
    for (int i = threadIdx.x; i < bwords; i += blockDim.x) bdst[i] = bsrc[i];
}

// Pipelined fused pass: warps 0-7 compute, warp 8 is the producer. The producer streams every
// tile of this CTA through a two-buffer ring: bulk loads complete on full[b]; when the compute
// warps have finished buffer b they arrive on empty[b]; the producer then bulk-stores it, waits
// for the store to have read shared memory, and loads the CTA's next-but-one tile into it. Loads,
// compute and stores of consecutive tiles overlap. Every wait is bounded.
constexpr int kPipeThreads = 288;

// CTAs per SM the kernels are compiled for. FP64 elements (complex128, real64) get the larger
// register budget: that path is bound by FP64 issue, not occupancy. Real32 tiles (32 KB, two per
// CTA) leave room for three pipelined CTAs per SM, and the latency-bound passes gain more from the
// third CTA's warps than they lose to the smaller register budget.
template <typename T>
constexpr int wide_regs() {
    return sizeof(typename Elem<T>::R) == 8 ? 1 : 0;
}
template <typename T>
constexpr int pipe_ctas() {
    return sizeof(T) == 4 ? 3 : 2 - wide_regs<T>();
}

// The pipelined pass loop, shared by the operator interpreter (k_tile_pipe) and by passes the
// host specializes at run time: `compute(tile, member)` runs on the 256 compute threads for every
// tile of this CTA; the producer warp streams the tiles. `pd` is the pass (in shared memory),
// buf0/buf1 the two tile buffers, full/empty the ring's mbarriers (initialised by the caller).
// With Swz, the tile moves in boxes of tensor copies through `tmap` with the 128-byte swizzle (the
// compute side addresses the tile through the same swizzle): a pass whose chunks are 512 bytes
// pairs chunks 2q and 2q+1 (they differ in register bit hi[0]) in one 3-D box of 1 KB; larger
// chunks move as 2-D boxes of min(chunk, 16 KB). Otherwise one plain bulk copy per chunk.
template <typename T, bool Swz = false, typename F>
__device__ __forceinline__ void pipe_run(T* __restrict__ state, int64_t member_elems, const PassDesc& pd, T* buf0,
                                         T* buf1, uint64_t* full, uint64_t* empty, int64_t tiles_per_member,
                                         int64_t total_tiles, int* status, F&& compute, const Tmap* tmap = nullptr,
                                         int64_t first = -1, int64_t stride = 0) {
    const int K = pd.K, L = pd.L;
    const int nchunks = 1 << (K - L);
    const uint32_t chunk_bytes = (uint32_t)(sizeof(T) << L);
    if (first < 0) {  // this CTA's tiles: blockIdx.x, then every gridDim.x-th (or a CTA range's own share)
        first = blockIdx.x;
        stride = gridDim.x;
    }
    // the pass's tensor map has this box shape (host jit_launch)
    const bool pair = chunk_bytes == 512u;
    const uint32_t box_bytes = pair ? 1024u : (chunk_bytes < 16384u ? chunk_bytes : 16384u);
    const int box_elems = (int)(box_bytes / sizeof(T));
    const int box_shift = (Swz && !pair) ? (__ffs((int)(chunk_bytes / box_bytes)) - 1) : 0;  // boxes per chunk
    const int nboxes = pair ? nchunks / 2 : nchunks << box_shift;
    const int h = pd.hi[0];  // the register bit between the two chunks of a pair
    if (threadIdx.x >= 256) {
        // ---------------- producer warp
        const int lane = threadIdx.x - 256;
        auto tile_at = [&](int64_t t, T** mem, uint64_t* base) {
            const int64_t member = t / tiles_per_member;
            const uint64_t tt = (uint64_t)(t - member * tiles_per_member);
            *mem = state + member * member_elems;
            *base = deposit(tt, pd.outer, pd.nouter) | pd.fix;
        };
        // the register element where box q of the tile at `mem + base` starts
        auto box_elem = [&](const T* mem, uint64_t base, int q) {
            const uint64_t c = pair ? 2 * (uint64_t)q : (uint64_t)(q >> box_shift);
            const uint64_t sub = pair ? 0 : (uint64_t)(q & ((1 << box_shift) - 1)) * (uint64_t)box_elems;
            return (uint64_t)(mem - state) + (base | deposit(c, pd.hi, K - L)) + sub;
        };
        // coordinates: 2-D (row of 128 bytes), 3-D (row within the 2^h-element block, block)
        auto copy_out = [&](uint64_t e, const T* src) {
            if (pair)
                tma_store_3d(tmap, (int)(((e & ((1ull << h) - 1)) * sizeof(T)) >> 7), (int)(e >> h), src);
            else
                tma_store_2d(tmap, (int)((e * sizeof(T)) >> 7), src);
        };
        auto copy_in = [&](uint64_t e, T* dst, uint64_t* bar) {
            if (pair)
                tma_load_3d(dst, tmap, (int)(((e & ((1ull << h) - 1)) * sizeof(T)) >> 7), (int)(e >> h), bar);
            else
                tma_load_2d(dst, tmap, (int)((e * sizeof(T)) >> 7), bar);
        };
        auto store = [&](int64_t t, T* buf) {
            T* mem;
            uint64_t base;
            tile_at(t, &mem, &base);
            if constexpr (Swz) {
                for (int q = lane; q < nboxes; q += 32) copy_out(box_elem(mem, base, q), buf + (size_t)q * box_elems);
            } else {
                for (int c = lane; c < nchunks; c += 32)
                    bulk_s2g(mem + (base | deposit((uint64_t)c, pd.hi, K - L)), buf + ((size_t)c << L), chunk_bytes);
            }
            bulk_commit();
            bulk_wait_read();
            __syncwarp();
        };
        int64_t it = 0;
        for (int64_t t = first; t < total_tiles; t += stride, ++it) {
            const int b = (int)(it & 1);
            T* buf = b ? buf1 : buf0;
            if (it >= 2) {  // buffer b still holds tile it-2: wait for its compute, store it
                const bool ok = mbar_wait_bounded(&empty[b], (uint32_t)(((it >> 1) - 1) & 1), status);
                if (!ok) {
                    bulk_wait_all();  // our own stores in flight, then leave
                    return;
                }
                store(t - 2 * stride, buf);
            }
            T* mem;
            uint64_t base;
            tile_at(t, &mem, &base);
            if (lane == 0) mbar_arrive_expect_tx(&full[b], chunk_bytes * (uint32_t)nchunks);
            __syncwarp();
            if constexpr (Swz) {
                for (int q = lane; q < nboxes; q += 32) copy_in(box_elem(mem, base, q), buf + (size_t)q * box_elems, &full[b]);
            } else {
                for (int c = lane; c < nchunks; c += 32)
                    bulk_g2s(buf + ((size_t)c << L), mem + (base | deposit((uint64_t)c, pd.hi, K - L)), chunk_bytes,
                             &full[b]);
            }
        }
        // the last one or two tiles
        const int64_t n_it = it;
        for (int64_t j = (n_it >= 2 ? n_it - 2 : 0); j < n_it; ++j) {
            const int b = (int)(j & 1);
            const bool ok = mbar_wait_bounded(&empty[b], (uint32_t)((j >> 1) & 1), status);
            if (!ok) {
                bulk_wait_all();
                return;
            }
            store(first + j * stride, b ? buf1 : buf0);
        }
        bulk_wait_all();
        return;
    }
    // ---------------- compute warps
    int64_t it = 0;
    for (int64_t t = first; t < total_tiles; t += stride, ++it) {
        const int b = (int)(it & 1);
        T* tile = b ? buf1 : buf0;
        const bool ok = mbar_wait_bounded(&full[b], (uint32_t)((it >> 1) & 1), status);
        if (cbar_or(!ok)) return;  // every compute thread leaves together on a timeout
        compute(tile, t / tiles_per_member);
        fence_proxy_async_smem();  // this thread's writes, before the producer's bulk store reads them
        mbar_arrive(&empty[b]);
    }
}

// Barriers of the two-buffer ring: `full` completes on the bulk loads, `empty` when all 256
// compute threads are done with the buffer.
__device__ __forceinline__ void pipe_init(uint64_t* full, uint64_t* empty) {
    if (threadIdx.x == 0) {
        mbar_init(&full[0], 1);
        mbar_init(&full[1], 1);
        mbar_init(&empty[0], 256);
        mbar_init(&empty[1], 256);
        fence_mbar_init();
    }
}

template <typename T>
__global__ void __launch_bounds__(kPipeThreads, pipe_ctas<T>()) k_tile_pipe(T* __restrict__ state, int64_t member_elems,
                                                               const PassDesc* __restrict__ pass_g,
                                                               const TileOp* __restrict__ ops,
                                                               const BlockDesc* __restrict__ blocks,
                                                               const T* __restrict__ data, int64_t tiles_per_member,
                                                               int64_t total_tiles, int* status, TrajCtx ctx) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ uint64_t full[2], empty[2];
    __shared__ PassDesc pd;
    const size_t tile_bytes = sizeof(T) << pass_g->K;
    T* buf0 = reinterpret_cast<T*>(smem_raw);
    T* buf1 = reinterpret_cast<T*>(smem_raw + tile_bytes);
    TileOp* sops = reinterpret_cast<TileOp*>(smem_raw + 2 * tile_bytes);
    BlockDesc* sblk = reinterpret_cast<BlockDesc*>(sops + pass_g->nops);
    OpRec* recs = reinterpret_cast<OpRec*>(sblk + pass_g->nblocks);
    if (threadIdx.x == 0) pd = *pass_g;
    stage_pass<T>(pass_g, ops, blocks, sops, sblk);
    pipe_init(full, empty);
    __syncthreads();
    pipe_run<T>(state, member_elems, pd, buf0, buf1, full, empty, tiles_per_member, total_tiles, status,
                [&](T* tile, int64_t member) { compute_tile<T>(tile, pd.K, pd, sblk, sops, recs, data, member, ctx); });
}

// One program's pass in a launch over several registers (circuits of uneven widths): the
// program's device arrays, its register, and the range of the launch's CTAs that work on it.
struct RaggedJob {
    void* state;
    int64_t member_elems;
    const PassDesc* pass;
    const TileOp* ops;
    const BlockDesc* blocks;
    const void* data;
    int64_t tiles_per_member, total_tiles;
    int cta0, ctas;  // CTAs cta0 .. cta0 + ctas - 1 of the launch take this job's tiles
};

// Pass k of every program of a ragged run in one launch: each CTA finds its job (jobs in CTA
// order), stages that pass's operators and runs the pipelined loop over its share of the job's
// tiles, exactly as k_tile_pipe does for one register.
template <typename T>
__global__ void __launch_bounds__(kPipeThreads, pipe_ctas<T>()) k_tile_pipe_ragged(const RaggedJob* __restrict__ jobs,
                                                                      int njobs, int* status) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ uint64_t full[2], empty[2];
    __shared__ PassDesc pd;
    __shared__ int job_s;
    if (threadIdx.x == 0) {
        int lo = 0, hi = njobs - 1;  // the last job whose first CTA is at or below this one
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (jobs[mid].cta0 <= (int)blockIdx.x) lo = mid;
            else hi = mid - 1;
        }
        job_s = lo;
    }
    __syncthreads();
    const RaggedJob& J = jobs[job_s];
    const PassDesc* pass_g = J.pass;
    const size_t tile_bytes = sizeof(T) << pass_g->K;
    T* buf0 = reinterpret_cast<T*>(smem_raw);
    T* buf1 = reinterpret_cast<T*>(smem_raw + tile_bytes);
    TileOp* sops = reinterpret_cast<TileOp*>(smem_raw + 2 * tile_bytes);
    BlockDesc* sblk = reinterpret_cast<BlockDesc*>(sops + pass_g->nops);
    OpRec* recs = reinterpret_cast<OpRec*>(sblk + pass_g->nblocks);
    if (threadIdx.x == 0) pd = *pass_g;
    stage_pass<T>(pass_g, J.ops, J.blocks, sops, sblk);
    pipe_init(full, empty);
    __syncthreads();
    const T* data = static_cast<const T*>(J.data);
    const TrajCtx ctx{};
    pipe_run<T>(static_cast<T*>(J.state), J.member_elems, pd, buf0, buf1, full, empty, J.tiles_per_member,
                J.total_tiles, status,
                [&](T* tile, int64_t member) { compute_tile<T>(tile, pd.K, pd, sblk, sops, recs, data, member, ctx); },
                nullptr, (int64_t)blockIdx.x - J.cta0, (int64_t)J.ctas);
}

// A pass specialized by the host: `Body::run(tile, data, member)` is generated straight-line code
// (compile-time block bits, operator kinds, positions and data offsets; no operator dispatch).
// With Swz the dynamic shared memory holds 1 KB more than the two tiles: the tiles start on a
// 1024-byte boundary (every 512-byte box then starts on a box boundary).
template <typename T, typename Body, bool Swz>
__device__ __forceinline__ void pipe_kernel(T* __restrict__ state, int64_t member_elems, const PassDesc* __restrict__ pass_g,
                                            const T* __restrict__ data, int64_t tiles_per_member, int64_t total_tiles,
                                            int* status, const Tmap* tmap) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    __shared__ uint64_t full[2], empty[2];
    __shared__ PassDesc pd;
    const size_t tile_bytes = sizeof(T) << pass_g->K;
    unsigned char* tiles = smem_raw + (Swz ? ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u) : 0u);
    T* buf0 = reinterpret_cast<T*>(tiles);
    T* buf1 = reinterpret_cast<T*>(tiles + tile_bytes);
    if (threadIdx.x == 0) pd = *pass_g;
    pipe_init(full, empty);
    __syncthreads();
    pipe_run<T, Swz>(state, member_elems, pd, buf0, buf1, full, empty, tiles_per_member, total_tiles, status,
                     [&](T* tile, int64_t member) { Body::run(tile, data, member); }, tmap);
}

// Runs of N consecutive elements between shared memory and registers (16-, 8- or 4-byte
// accesses by size), for specialized passes whose group offsets are compile-time constants.
template <typename T, int N>
__device__ __forceinline__ void ld_run(const T* p, T* v) {
    if constexpr (sizeof(T) * N == 16 && sizeof(T) == 4) {
        const float4 w = *reinterpret_cast<const float4*>(p);
        v[0] = w.x, v[1] = w.y, v[2] = w.z, v[3] = w.w;
    } else if constexpr (sizeof(T) * N == 8 && sizeof(T) == 4) {
        const float2 w = *reinterpret_cast<const float2*>(p);
        v[0] = w.x, v[1] = w.y;
    } else if constexpr (sizeof(T) * N == 16 && sizeof(T) == 8) {
        const uint4 w = *reinterpret_cast<const uint4*>(p);
        memcpy(&v[0], &w.x, 8);
        memcpy(&v[1], &w.z, 8);
    } else {
#pragma unroll
        for (int i = 0; i < N; ++i) v[i] = p[i];
    }
}

// Two consecutive elements into (a, b) and back: the same tile offset of two neighbouring groups.
template <typename T>
__device__ __forceinline__ void ld_split(const T* p, T& a, T& b) {
    if constexpr (sizeof(T) == 4) {
        const float2 w = *reinterpret_cast<const float2*>(p);
        memcpy(&a, &w.x, 4);
        memcpy(&b, &w.y, 4);
    } else if constexpr (sizeof(T) == 8) {
        const uint4 w = *reinterpret_cast<const uint4*>(p);
        memcpy(&a, &w.x, 8);
        memcpy(&b, &w.z, 8);
    } else {
        a = p[0], b = p[1];
    }
}

template <typename T>
__device__ __forceinline__ void st_split(T* p, const T& a, const T& b) {
    if constexpr (sizeof(T) == 4) {
        float2 w;
        memcpy(&w.x, &a, 4);
        memcpy(&w.y, &b, 4);
        *reinterpret_cast<float2*>(p) = w;
    } else if constexpr (sizeof(T) == 8) {
        uint4 w;
        memcpy(&w.x, &a, 8);
        memcpy(&w.z, &b, 8);
        *reinterpret_cast<uint4*>(p) = w;
    } else {
        p[0] = a, p[1] = b;
    }
}

template <typename T, int N>
__device__ __forceinline__ void st_run(T* p, const T* v) {
    if constexpr (sizeof(T) * N == 16 && sizeof(T) == 4) {
        *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
    } else if constexpr (sizeof(T) * N == 8 && sizeof(T) == 4) {
        *reinterpret_cast<float2*>(p) = make_float2(v[0], v[1]);
    } else if constexpr (sizeof(T) * N == 16 && sizeof(T) == 8) {
        uint4 w;
        memcpy(&w.x, &v[0], 8);
        memcpy(&w.z, &v[1], 8);
        *reinterpret_cast<uint4*>(p) = w;
    } else {
#pragma unroll
        for (int i = 0; i < N; ++i) p[i] = v[i];
    }
}

// One fused pass over every tile of every member. Tiles are visited grid-stride; each CTA
// handles one tile at a time (CTAs co-resident on an SM overlap each other's copies).
template <typename T>
__global__ void __launch_bounds__(256, 3 - wide_regs<T>()) k_tile_pass(T* __restrict__ state, int64_t member_elems,
                                                   const PassDesc* __restrict__ pass_g,
                                                   const TileOp* __restrict__ ops, const BlockDesc* __restrict__ blocks,
                                                   const T* __restrict__ data, int64_t tiles_per_member,
                                                   int64_t total_tiles, int* status, TrajCtx ctx) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ uint64_t bar;
    __shared__ PassDesc pd;
    T* tile = reinterpret_cast<T*>(smem_raw);
    TileOp* sops = reinterpret_cast<TileOp*>(smem_raw + (sizeof(T) << pass_g->K));
    BlockDesc* sblk = reinterpret_cast<BlockDesc*>(sops + pass_g->nops);
    OpRec* recs = reinterpret_cast<OpRec*>(sblk + pass_g->nblocks);
    if (threadIdx.x == 0) pd = *pass_g;
    {
        // stage this pass's operators and blocks in shared memory (the same for every tile)
        const int nops = pass_g->nops;
        const int* src = reinterpret_cast<const int*>(ops + pass_g->first_op);
        int* dst = reinterpret_cast<int*>(sops);
        const int words = nops * (int)(sizeof(TileOp) / sizeof(int));
        for (int i = threadIdx.x; i < words; i += blockDim.x) dst[i] = src[i];
        const int* bsrc = reinterpret_cast<const int*>(blocks + pass_g->first_block);
        int* bdst = reinterpret_cast<int*>(sblk);
        const int bwords = pass_g->nblocks * (int)(sizeof(BlockDesc) / sizeof(int));
        for (int i = threadIdx.x; i < bwords; i += blockDim.x) bdst[i] = bsrc[i];
    }
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    const int K = pd.K, L = pd.L;
    const int nchunks = 1 << (K - L);
    const uint32_t chunk_bytes = (uint32_t)(sizeof(T) << L);
    const bool use_bulk = (chunk_bytes % 16) == 0;
    uint32_t parity = 0;
    for (int64_t t = blockIdx.x; t < total_tiles; t += gridDim.x) {
        const int64_t member = t / tiles_per_member;
        const uint64_t tt = (uint64_t)(t - member * tiles_per_member);
        T* mem = state + member * member_elems;
        const uint64_t base = deposit(tt, pd.outer, pd.nouter) | pd.fix;
        // ---- load
        if (use_bulk) {
            if (threadIdx.x < 32) {
                if (threadIdx.x == 0) mbar_arrive_expect_tx(&bar, chunk_bytes * (uint32_t)nchunks);
                __syncwarp();
                for (int c = threadIdx.x; c < nchunks; c += 32)
                    bulk_g2s(tile + ((size_t)c << L), mem + (base | deposit((uint64_t)c, pd.hi, K - L)), chunk_bytes,
                             &bar);
            }
            const bool ok = mbar_wait_bounded(&bar, parity, status);
            if (__syncthreads_or(!ok)) return;  // every thread leaves together on a timeout
            parity ^= 1;
        } else {
            const int n = 1 << K;
            for (int i = threadIdx.x; i < n; i += blockDim.x) {
                uint64_t g = base | deposit((uint64_t)(i >> L), pd.hi, K - L) | (uint64_t)(i & ((1 << L) - 1));
                tile[i] = mem[g];
            }
        }
        // ---- compute: register blocks, or one shared-memory operator for a wide block
        __syncthreads();
        compute_tile<T>(tile, K, pd, sblk, sops, recs, data, member, ctx);
        __syncthreads();
        // ---- store
        if (use_bulk) {
            fence_proxy_async_smem();
            __syncthreads();
            if (threadIdx.x < 32) {
                for (int c = threadIdx.x; c < nchunks; c += 32)
                    bulk_s2g(mem + (base | deposit((uint64_t)c, pd.hi, K - L)), tile + ((size_t)c << L), chunk_bytes);
                bulk_commit();
                bulk_wait_read();
            }
            __syncthreads();
        } else {
            const int n = 1 << K;
            for (int i = threadIdx.x; i < n; i += blockDim.x) {
                uint64_t g = base | deposit((uint64_t)(i >> L), pd.hi, K - L) | (uint64_t)(i & ((1 << L) - 1));
                mem[g] = tile[i];
            }
            __syncthreads();
        }
    }
    if (use_bulk && threadIdx.x < 32) bulk_wait_all();
}


}  // namespace lsg
