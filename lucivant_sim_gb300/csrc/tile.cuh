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

template <typename R>
__device__ __forceinline__ Cx<R> ldm(const Cx<R>* m, int i) {
    return m[i];
}

// 1-bit dense: the common case (fused one-qubit gates; one-qubit density superoperators use 2).
template <typename R>
__device__ __forceinline__ void dense1(Cx<R>* t, int tbits, int b, const Cx<R>* m) {
    const Cx<R> m00 = m[0], m01 = m[1], m10 = m[2], m11 = m[3];
    const int groups = 1 << (tbits - 1);
    for (int g = threadIdx.x; g < groups; g += blockDim.x) {
        const uint32_t i0 = ins0((uint32_t)g, b), i1 = i0 | (1u << b);
        const Cx<R> a0 = t[i0], a1 = t[i1];
        t[i0] = cfma(m01, a1, cmul(m00, a0));
        t[i1] = cfma(m11, a1, cmul(m10, a0));
    }
}

// 2-bit dense on (hi_bit = matrix MSB b0, b1); lo/hi are the sorted positions.
template <typename R>
__device__ __forceinline__ void dense2(Cx<R>* t, int tbits, int b0, int b1, const Cx<R>* m) {
    const int lo = min(b0, b1), hi = max(b0, b1);
    const uint32_t o1 = 1u << b1, o2 = 1u << b0;
    const int groups = 1 << (tbits - 2);
    for (int g = threadIdx.x; g < groups; g += blockDim.x) {
        const uint32_t base = ins0(ins0((uint32_t)g, lo), hi);
        const Cx<R> v0 = t[base], v1 = t[base | o1], v2 = t[base | o2], v3 = t[base | o1 | o2];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            Cx<R> acc = cmul(ldm(m, 4 * r), v0);
            acc = cfma(ldm(m, 4 * r + 1), v1, acc);
            acc = cfma(ldm(m, 4 * r + 2), v2, acc);
            acc = cfma(ldm(m, 4 * r + 3), v3, acc);
            const uint32_t at = base | ((r & 1) ? o1 : 0u) | ((r & 2) ? o2 : 0u);
            t[at] = acc;
        }
    }
}

template <typename R>
__device__ __forceinline__ Cx<R> pick4(const Cx<R>& v0, const Cx<R>& v1, const Cx<R>& v2, const Cx<R>& v3, int s) {
    const Cx<R> a = (s & 1) ? v1 : v0;
    const Cx<R> b = (s & 1) ? v3 : v2;
    return (s & 2) ? b : a;
}

// permutations with phases on 1 or 2 bits (x, cx, swap and their phased forms)
template <typename R>
__device__ __forceinline__ void perm1(Cx<R>* t, int tbits, int b, const Cx<R>* m) {
    const Cx<R> p0 = m[0], p1 = m[1];
    const int s0 = (int)m[2].re;
    const int groups = 1 << (tbits - 1);
    for (int g = threadIdx.x; g < groups; g += blockDim.x) {
        const uint32_t i0 = ins0((uint32_t)g, b), i1 = i0 | (1u << b);
        const Cx<R> a0 = t[i0], a1 = t[i1];
        t[i0] = cmul(p0, s0 ? a1 : a0);
        t[i1] = cmul(p1, s0 ? a0 : a1);
    }
}

template <typename R>
__device__ __forceinline__ void perm2(Cx<R>* t, int tbits, int b0, int b1, const Cx<R>* m) {
    const int lo = min(b0, b1), hi = max(b0, b1);
    const uint32_t o1 = 1u << b1, o2 = 1u << b0;
    const Cx<R> p0 = m[0], p1 = m[1], p2 = m[2], p3 = m[3];
    const int s0 = (int)m[4].re, s1 = (int)m[5].re, s2 = (int)m[6].re, s3 = (int)m[7].re;
    const int groups = 1 << (tbits - 2);
    for (int g = threadIdx.x; g < groups; g += blockDim.x) {
        const uint32_t base = ins0(ins0((uint32_t)g, lo), hi);
        const Cx<R> v0 = t[base], v1 = t[base | o1], v2 = t[base | o2], v3 = t[base | o1 | o2];
        t[base] = cmul(p0, pick4(v0, v1, v2, v3, s0));
        t[base | o1] = cmul(p1, pick4(v0, v1, v2, v3, s1));
        t[base | o2] = cmul(p2, pick4(v0, v1, v2, v3, s2));
        t[base | o1 | o2] = cmul(p3, pick4(v0, v1, v2, v3, s3));
    }
}

// Wide operators (3 to 5 bits): rare (Toffoli-class gates, two-qubit Kraus superoperators), kept
// out of line so their register needs don't shape the common path.
template <typename R>
__device__ __noinline__ void wide_op(Cx<R>* t, int tbits, int kind, int k, const int* lb, const int* sorted,
                                     const Cx<R>* m) {
    const int D = 1 << k;
    uint32_t offs[32];
    Cx<R> v[32];
    for (int j = 0; j < D; ++j) {
        uint32_t o = 0;
        for (int i = 0; i < k; ++i) o |= (uint32_t)((j >> (k - 1 - i)) & 1) << lb[i];
        offs[j] = o;
    }
    const int groups = 1 << (tbits - k);
    for (int g = threadIdx.x; g < groups; g += blockDim.x) {
        uint32_t base = (uint32_t)g;
        for (int i = 0; i < k; ++i) base = ins0(base, sorted[i]);
        for (int j = 0; j < D; ++j) v[j] = t[base | offs[j]];
        if (kind == LSG_OP_MATRIX) {
            for (int r = 0; r < D; ++r) {
                Cx<R> acc;
                for (int c = 0; c < D; ++c) acc = cfma(m[r * D + c], v[c], acc);
                t[base | offs[r]] = acc;
            }
        } else {
            for (int r = 0; r < D; ++r) t[base | offs[r]] = cmul(m[r], v[(int)m[D + r].re]);
        }
    }
}

template <typename R>
__device__ __forceinline__ void op_diag(Cx<R>* tile, int tbits, int k, const int* lb, const Cx<R>* m) {
    const int n = 1 << tbits;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        int j = 0;
        for (int b = 0; b < k; ++b) j = (j << 1) | ((i >> lb[b]) & 1);
        tile[i] = cmul(m[j], tile[i]);
    }
}

template <typename R>
__device__ __forceinline__ void op_scale(Cx<R>* tile, int tbits, const Cx<R>* m) {
    const int n = 1 << tbits;
    const Cx<R> f = m[0];
    for (int i = threadIdx.x; i < n; i += blockDim.x) tile[i] = cmul(f, tile[i]);
}

// (1-p) rho + (p/d) I (x) Tr_t(rho) on kq row bits then kq column bits (kq = 1 or 2).
template <typename R, int KQ>
__device__ __forceinline__ void op_depol(Cx<R>* t, int tbits, const int* lb, const int* sorted, const Cx<R>* m) {
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
    for (int g = threadIdx.x; g < groups; g += blockDim.x) {
        uint32_t base = (uint32_t)g;
#pragma unroll
        for (int i = 0; i < KB; ++i) base = ins0(base, srt[i]);
        Cx<R> tr;
#pragma unroll
        for (int s = 0; s < d; ++s) {
            const int j = (s << KQ) | s;
            uint32_t o = 0;
#pragma unroll
            for (int i = 0; i < KB; ++i) o |= (uint32_t)((j >> (KB - 1 - i)) & 1) << l[i];
            const Cx<R> v = t[base | o];
            tr.re += v.re;
            tr.im += v.im;
        }
#pragma unroll
        for (int j = 0; j < D; ++j) {
            uint32_t o = 0;
#pragma unroll
            for (int i = 0; i < KB; ++i) o |= (uint32_t)((j >> (KB - 1 - i)) & 1) << l[i];
            const Cx<R> v = t[base | o];
            Cx<R> out(v.re * keep, v.im * keep);
            if ((j >> KQ) == (j & (d - 1))) {
                out.re += share * tr.re;
                out.im += share * tr.im;
            }
            t[base | o] = out;
        }
    }
}

// A state-independent noise channel in a trajectory: the member picks branch i, the first with
// u < cum[i] (cum = running sums of the branch probabilities, as engines.py:163-171 accumulates
// them), and applies that branch's unitary unless it is the identity. Data: `count` entries
// (re = cumulative probability, im = 1 for an identity branch), then `count` dense 2^k matrices.
template <typename R>
__device__ __forceinline__ void op_mixture(Cx<R>* t, int tbits, const TileOp& op, const Cx<R>* m, double u) {
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
    const Cx<R>* mat = m + nb + (int64_t)pick * d * d;
    if (op.k == 1) dense1<R>(t, tbits, op.lb[0], mat);
    else if (op.k == 2) dense2<R>(t, tbits, op.lb[0], op.lb[1], mat);
    else wide_op<R>(t, tbits, LSG_OP_MATRIX, op.k, op.lb, op.sorted, mat);
}

template <typename R>
__device__ void run_ops(Cx<R>* tile, int tbits, const TileOp* __restrict__ ops, int nops,
                        const Cx<R>* __restrict__ data, int64_t member, const TrajCtx& ctx) {
    const uint64_t pred = ctx.u ? ctx.pred[member] : ~0ull;
    const int64_t cur = ctx.u ? ctx.cursor[member] : 0;
    for (int o = 0; o < nops; ++o) {
        const TileOp& op = ops[o];  // staged in shared memory
        const int kind = op.kind, k = op.k;
        const Cx<R>* m = data + op.data + member * op.stride;
        if (!((pred >> op.pred) & 1)) continue;  // a branch this member did not take (CTA-uniform)
        __syncthreads();
        if (kind == kOpMixture) {
            op_mixture<R>(tile, tbits, op, m, ctx.u[member * ctx.ustride + cur + op.draw]);
        } else if (kind == LSG_OP_MATRIX && k == 1) {
            dense1<R>(tile, tbits, op.lb[0], m);
        } else if (kind == LSG_OP_MATRIX && k == 2) {
            dense2<R>(tile, tbits, op.lb[0], op.lb[1], m);
        } else if (kind == LSG_OP_PERM && k == 1) {
            perm1<R>(tile, tbits, op.lb[0], m);
        } else if (kind == LSG_OP_PERM && k == 2) {
            perm2<R>(tile, tbits, op.lb[0], op.lb[1], m);
        } else if (kind == LSG_OP_DIAG) {
            op_diag<R>(tile, tbits, k, op.lb, m);
        } else if (kind == LSG_OP_DEPOL) {
            if (k == 2) op_depol<R, 1>(tile, tbits, op.lb, op.sorted, m);
            else op_depol<R, 2>(tile, tbits, op.lb, op.sorted, m);
        } else if (kind == LSG_OP_SCALE) {
            op_scale<R>(tile, tbits, m);
        } else {
            wide_op<R>(tile, tbits, kind, k, op.lb, op.sorted, m);
        }
    }
    __syncthreads();
}

// One fused pass over every tile of every member. Tiles are visited grid-stride; each CTA
// handles one tile at a time (CTAs co-resident on an SM overlap each other's copies).
template <typename R>
__global__ void __launch_bounds__(256, sizeof(R) == 4 ? 4 : 3) k_tile_pass(Cx<R>* __restrict__ state, int64_t member_elems,
                                                   const PassDesc* __restrict__ pass_g,
                                                   const TileOp* __restrict__ ops,
                                                   const Cx<R>* __restrict__ data, int64_t tiles_per_member,
                                                   int64_t total_tiles, int* status, TrajCtx ctx) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ uint64_t bar;
    __shared__ PassDesc pd;
    Cx<R>* tile = reinterpret_cast<Cx<R>*>(smem_raw);
    TileOp* sops = reinterpret_cast<TileOp*>(smem_raw + (sizeof(Cx<R>) << pass_g->K));
    if (threadIdx.x == 0) pd = *pass_g;
    {
        // stage this pass's operators in shared memory (the same for every tile of the pass)
        const int nops = pass_g->nops;
        const int* src = reinterpret_cast<const int*>(ops + pass_g->first_op);
        int* dst = reinterpret_cast<int*>(sops);
        const int words = nops * (int)(sizeof(TileOp) / sizeof(int));
        for (int i = threadIdx.x; i < words; i += blockDim.x) dst[i] = src[i];
    }
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    const int K = pd.K, L = pd.L;
    const int nchunks = 1 << (K - L);
    const uint32_t chunk_bytes = (uint32_t)(sizeof(Cx<R>) << L);
    const bool use_bulk = (chunk_bytes % 16) == 0;
    uint32_t parity = 0;
    for (int64_t t = blockIdx.x; t < total_tiles; t += gridDim.x) {
        const int64_t member = t / tiles_per_member;
        const uint64_t tt = (uint64_t)(t - member * tiles_per_member);
        Cx<R>* mem = state + member * member_elems;
        const uint64_t base = deposit(tt, pd.outer, pd.nouter);
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
        // ---- compute
        run_ops<R>(tile, K, sops, pd.nops, data, member, ctx);
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
