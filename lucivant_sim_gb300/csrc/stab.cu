// The stabilizer engine (Orrery's src/lucivant_sim/stabilizer.py) on the device.
//
//  * Tableau: x, z bit-packed qubit-major — word w of qubit q holds rows 32w..32w+31 — and the
//    sign bits r; rows 0..n-1 destabilizers, n..2n-1 stabilizers (stabilizer.py:193-208). Gates
//    are applied moment by moment (gates of a moment act on disjoint qubits): one CTA per 32-row
//    word column keeps that column of x and z in shared memory and its threads take the gates of
//    a moment in parallel; sign updates are XOR-combined. Named gates use the update rules of
//    stabilizer.py:224-254, other Clifford gates the conjugation table (:256-264).
//  * support(): GF(2) elimination on the stabilizer rows packed row-major in 64-bit words, with
//    the reference's pivot rule (first unused row with the bit set, qubits ascending) and the
//    popcount phase arithmetic of _rowsum_packed (stabilizer.py:333-395); then the Z constraints
//    (:398-422) and, for a subset of qubits, the row basis (:425-440).
//  * Pauli frames (stabilizer.py:514-563): one CTA per 32-shot word keeps every qubit's frame
//    word in shared memory; noise branches come from a device PCG64 that regenerates the run's
//    NumPy stream bit for bit (128-bit LCG, XSL-RR output, jump-ahead), so counts are identical.
//  * Ideal sampling (stabilizer.py:597-619): x0 plus combinations of the basis picked by the
//    same stream's uint8 integers.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "common.cuh"

namespace lsg {

typedef unsigned __int128 u128;

__host__ __device__ __forceinline__ u128 pcg_mult() {
    return ((u128)0x2360ED051FC65DA4ull << 64) | (u128)0x4385DF649FCCF645ull;
}

__host__ __device__ __forceinline__ uint64_t pcg_output(u128 s) {
    const uint64_t hi = (uint64_t)(s >> 64), lo = (uint64_t)s;
    const uint64_t x = hi ^ lo;
    const unsigned r = (unsigned)(hi >> 58);
    return (x >> r) | (x << ((64 - r) & 63));
}

// jump coefficients: advancing by delta steps maps s to mult * s + plus (Brown, "Random number
// generation with arbitrary strides", 1994)
__host__ __device__ inline void pcg_jump(u128 inc, uint64_t delta, u128* mult, u128* plus) {
    u128 am = 1, ap = 0, cm = pcg_mult(), cp = inc;
    while (delta > 0) {
        if (delta & 1) {
            am *= cm;
            ap = ap * cm + cp;
        }
        cp = (cm + 1) * cp;
        cm *= cm;
        delta >>= 1;
    }
    *mult = am;
    *plus = ap;
}

__host__ __device__ inline u128 pcg_advance(u128 s, u128 inc, uint64_t delta) {
    u128 m, p;
    pcg_jump(inc, delta, &m, &p);
    return m * s + p;
}

// raw draw number i (0-based) of a generator whose current state is s
__host__ __device__ inline uint64_t pcg_raw(u128 s, u128 inc, uint64_t i) { return pcg_output(pcg_advance(s, inc, i + 1)); }

__host__ __device__ __forceinline__ double pcg_double(uint64_t raw) { return (double)(raw >> 11) * (1.0 / 9007199254740992.0); }

// the uint8 integers(0, 2) value number t of a run that starts with no buffered uint32: the top
// bit of byte t%4 of uint32 number t/4; uint32 2j is the low half of raw j, 2j+1 the high half
__host__ __device__ inline int pcg_bit_at(u128 s, u128 inc, uint64_t t) {
    const uint64_t raw = pcg_raw(s, inc, t >> 3);
    const uint32_t word = ((t >> 2) & 1) ? (uint32_t)(raw >> 32) : (uint32_t)raw;
    return (word >> (8 * (t & 3) + 7)) & 1;
}

constexpr int kS = 256;

struct GateRec {  // lsg_cgate on the device
    int16_t code, noise, a, b, c, pad;
    int32_t nk;  // index among the noisy gates (frames), -1 if none
};

struct CTable {  // a generic Clifford conjugation table
    int32_t k, pad;
    uint8_t e[64];  // (sign << 7) | image bits, index = Pauli bits (x0 z0 x1 z1 ...), first qubit MSB
};

struct NTable {  // Pauli noise branches: normalised cumulative probabilities and labels
    int32_t k, nb;
    double cum[16];
    uint8_t label[16];  // per qubit i (first qubit bit 2(k-1-i)): x bit then z bit
    // cum[i] <= u for a uniform u = m * 2^-53 (m = raw >> 11) exactly when m >= thr[i] =
    // ceil(cum[i] * 2^53): the branch search in integers, with the same answers
    uint64_t thr[16];
};

__device__ __forceinline__ uint32_t xor_reduce_block(uint32_t v) {
    __shared__ uint32_t red[32];
    for (int off = 16; off > 0; off >>= 1) v ^= __shfl_xor_sync(0xffffffffu, v, off);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    uint32_t out = 0;
    if (threadIdx.x == 0)
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) out ^= red[i];
    __syncthreads();
    return out;
}

// apply one gate to one 32-row word column held in X, Z (shared); returns the sign flips
__device__ __forceinline__ uint32_t tab_gate(uint32_t* X, uint32_t* Z, const GateRec& g, const CTable* tables) {
    const int a = g.a;
    uint32_t r = 0;
    switch (g.code) {
        case 0: break;
        case 1: {  // h
            const uint32_t x = X[a], z = Z[a];
            r = x & z;
            X[a] = z;
            Z[a] = x;
            break;
        }
        case 2: r = X[a] & Z[a]; Z[a] ^= X[a]; break;   // s
        case 3: r = X[a] & ~Z[a]; Z[a] ^= X[a]; break;  // sdg
        case 4: r = Z[a]; break;                        // x
        case 5: r = X[a] ^ Z[a]; break;                 // y
        case 6: r = X[a]; break;                        // z
        case 7: {                                       // cx a -> b
            const int b = g.b;
            r = X[a] & Z[b] & ~(X[b] ^ Z[a]);
            X[b] ^= X[a];
            Z[a] ^= Z[b];
            break;
        }
        case 8: {  // cz
            const int b = g.b;
            r = X[a] & X[b] & (Z[a] ^ Z[b]);
            Z[a] ^= X[b];
            Z[b] ^= X[a];
            break;
        }
        default: {  // conjugation table, row by row
            const CTable& t = tables[g.code - 16];
            const int k = t.k;
            const int q[3] = {g.a, g.b, g.c};
            uint32_t nx[3] = {0, 0, 0}, nz[3] = {0, 0, 0};
            for (int j = 0; j < 32; ++j) {
                int idx = 0;
                for (int i = 0; i < k; ++i) idx = (idx << 2) | (((X[q[i]] >> j) & 1) << 1) | ((Z[q[i]] >> j) & 1);
                const uint8_t e = t.e[idx];
                r |= (uint32_t)(e >> 7) << j;
                for (int i = 0; i < k; ++i) {
                    nx[i] |= (uint32_t)((e >> (2 * (k - 1 - i) + 1)) & 1) << j;
                    nz[i] |= (uint32_t)((e >> (2 * (k - 1 - i))) & 1) << j;
                }
            }
            for (int i = 0; i < k; ++i) {
                X[q[i]] = nx[i];
                Z[q[i]] = nz[i];
            }
            break;
        }
    }
    return r;
}

// frames: conjugation without signs (stabilizer.py:566-594)
__device__ __forceinline__ void frame_gate(uint32_t* X, uint32_t* Z, const GateRec& g, const CTable* tables) {
    const int a = g.a;
    switch (g.code) {
        case 0: case 4: case 5: case 6: break;
        case 1: {
            const uint32_t x = X[a];
            X[a] = Z[a];
            Z[a] = x;
            break;
        }
        case 2: case 3: Z[a] ^= X[a]; break;
        case 7: X[g.b] ^= X[a]; Z[a] ^= Z[g.b]; break;
        case 8: Z[a] ^= X[g.b]; Z[g.b] ^= X[a]; break;
        default: tab_gate(X, Z, g, tables); break;  // the table's sign output is ignored
    }
}

// Tableau: one CTA per 32-row column; gates of a moment in parallel.
__global__ void k_tab_apply(uint32_t* __restrict__ xg, uint32_t* __restrict__ zg, uint32_t* __restrict__ rg, int n, int words,
                            const GateRec* __restrict__ gates, const int64_t* __restrict__ moments, int64_t nmoments,
                            const CTable* __restrict__ tables) {
    extern __shared__ uint32_t sm[];
    uint32_t* X = sm;
    uint32_t* Z = sm + n;
    const int w = blockIdx.x;
    for (int q = threadIdx.x; q < n; q += blockDim.x) {
        X[q] = xg[(int64_t)q * words + w];
        Z[q] = zg[(int64_t)q * words + w];
    }
    __syncthreads();
    uint32_t racc = 0;
    for (int64_t m = 0; m < nmoments; ++m) {
        const int64_t lo = moments[m], hi = moments[m + 1];
        for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) racc ^= tab_gate(X, Z, gates[i], tables);
        __syncthreads();
    }
    const uint32_t flips = xor_reduce_block(racc);
    for (int q = threadIdx.x; q < n; q += blockDim.x) {
        xg[(int64_t)q * words + w] = X[q];
        zg[(int64_t)q * words + w] = Z[q];
    }
    if (threadIdx.x == 0) rg[w] ^= flips;
}

// stabilizer rows n..2n-1 to row-major 64-bit words: sx[i * W + v] bit j = x[64v + j][n + i]
__global__ void k_tab_rows(const uint32_t* __restrict__ xg, const uint32_t* __restrict__ zg, const uint32_t* __restrict__ rg,
                           int n, int words, int W, uint64_t* sx, uint64_t* sz, uint8_t* sr) {
    const int64_t total = (int64_t)n * W;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(t / W), v = (int)(t % W);
        const int row = n + i;
        uint64_t bx = 0, bz = 0;
        for (int j = 0; j < 64; ++j) {
            const int q = 64 * v + j;
            if (q >= n) break;
            bx |= (uint64_t)((xg[(int64_t)q * words + (row >> 5)] >> (row & 31)) & 1) << j;
            bz |= (uint64_t)((zg[(int64_t)q * words + (row >> 5)] >> (row & 31)) & 1) << j;
        }
        sx[t] = bx;
        sz[t] = bz;
        if (v == 0) sr[i] = (rg[row >> 5] >> (row & 31)) & 1;
    }
}

// pivot for column q: the first row with bit q set that is not used (rows in index order)
__global__ void k_elim_pivot(const uint64_t* __restrict__ mat, int rows, int W, int q, uint8_t* used, int* pivot,
                             int* pivots, int* npiv, int use_flags) {
    __shared__ int best;
    if (threadIdx.x == 0) best = 0x7fffffff;
    __syncthreads();
    for (int i = threadIdx.x; i < rows; i += blockDim.x)
        if (((mat[(int64_t)i * W + (q >> 6)] >> (q & 63)) & 1) && !(use_flags && used[i])) atomicMin(&best, i);
    __syncthreads();
    if (threadIdx.x == 0) {
        if (best == 0x7fffffff) {
            *pivot = -1;
        } else {
            *pivot = best;
            if (use_flags) used[best] = 1;
            pivots[*npiv] = best;
            *npiv += 1;
        }
    }
}

// rowsum of the pivot row into every other row with bit q set (a warp per row), with the phase
// exponent summed mod 4 from popcounts (stabilizer.py:381-395)
__global__ void k_sup_rowsum(uint64_t* __restrict__ sx, uint64_t* __restrict__ sz, uint8_t* __restrict__ sr, int rows, int W,
                             int q, const int* pivot) {
    const int p = *pivot;
    if (p < 0) return;
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int t = warp; t < rows; t += nwarps) {
        if (t == p || !((sx[(int64_t)t * W + (q >> 6)] >> (q & 63)) & 1)) continue;
        int g = 0;
        for (int v = lane; v < W; v += 32) {
            const uint64_t x1 = sx[(int64_t)p * W + v], z1 = sz[(int64_t)p * W + v];
            const uint64_t x2 = sx[(int64_t)t * W + v], z2 = sz[(int64_t)t * W + v];
            const uint64_t plus = (x1 & z1 & ~x2 & z2) | (x1 & ~z1 & x2 & z2) | (~x1 & z1 & x2 & ~z2);
            const uint64_t minus = (x1 & z1 & x2 & ~z2) | (x1 & ~z1 & ~x2 & z2) | (~x1 & z1 & x2 & z2);
            g += __popcll(plus) - __popcll(minus);
        }
        for (int off = 16; off > 0; off >>= 1) g += __shfl_xor_sync(0xffffffffu, g, off);
        __syncwarp();
        for (int v = lane; v < W; v += 32) {
            sx[(int64_t)t * W + v] ^= sx[(int64_t)p * W + v];
            sz[(int64_t)t * W + v] ^= sz[(int64_t)p * W + v];
        }
        if (lane == 0) {
            const long long total = 2ll * sr[t] + 2ll * sr[p] + g;
            sr[t] = (((total % 4) + 4) % 4) == 2 ? 1 : 0;
        }
    }
}

// plain elimination (no phase): every other row with bit q ^= the pivot row, and its
// right-hand side with it (stabilizer.py:405-419)
__global__ void k_elim_xor(uint64_t* __restrict__ m, uint8_t* __restrict__ rhs, int rows, int W, int q, const int* pivot) {
    const int p = *pivot;
    if (p < 0) return;
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int t = warp; t < rows; t += nwarps) {
        if (t == p || !((m[(int64_t)t * W + (q >> 6)] >> (q & 63)) & 1)) continue;
        __syncwarp();
        for (int v = lane; v < W; v += 32) m[(int64_t)t * W + v] ^= m[(int64_t)p * W + v];
        if (lane == 0 && rhs) rhs[t] ^= rhs[p];
    }
}

// ---- support() in one launch: a thread-block cluster holds the n stabilizer rows in its CTAs'
// shared memory (rows split evenly over the CTAs, a contiguous run of rows per warp) and walks
// the columns with one cluster barrier each. Per column every warp offers its lowest eligible row
// (atomicMin into its CTA's candidate slot), the cluster's minimum is read from every CTA's slot
// over distributed shared memory, each warp loads the pivot row from the owning CTA into
// registers and combines it into its own rows that have the bit. The X phase (pivots with the
// phase rowsum, stabilizer.py:371-395) is followed by the Z phase on the rows no X pivot took
// (plain GF(2) elimination with the signs as right-hand side, stabilizer.py:398-422).

__device__ __forceinline__ void cluster_barrier() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
__device__ __forceinline__ int cluster_ctarank() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return (int)r;
}
__device__ __forceinline__ int cluster_nctarank() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
    return (int)r;
}
// the address of `p` (this CTA's shared memory) in CTA `rank` of the cluster
__device__ __forceinline__ uint32_t dsmem_map(const void* p, int rank) {
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
    return r;
}
__device__ __forceinline__ uint64_t dsmem_u64(uint32_t a) {
    uint64_t v;
    asm volatile("ld.shared::cluster.u64 %0, [%1];" : "=l"(v) : "r"(a) : "memory");
    return v;
}
__device__ __forceinline__ int dsmem_s32(uint32_t a) {
    int v;
    asm volatile("ld.shared::cluster.s32 %0, [%1];" : "=r"(v) : "r"(a) : "memory");
    return v;
}
__device__ __forceinline__ int dsmem_u8(uint32_t a) {
    unsigned v;
    asm volatile("ld.shared::cluster.u8 %0, [%1];" : "=r"(v) : "r"(a) : "memory");
    return (int)v;
}

constexpr int kSupThreads = 1024;
constexpr int kSupWarps = kSupThreads / 32;
constexpr int kSupMaxCluster = 8;
constexpr int kSupRowsPerCta = 256;

struct SupArgs {
    uint64_t* sx;  // n rows x W words, row-major: in, the stabilizer rows; out, reduced
    uint64_t* sz;
    uint8_t* sr;
    uint8_t* used;  // out: rows taken as X pivots
    int* pivots;    // out: the X pivot rows in column order
    int* zcol;      // out: Z pivots, (column, row) in column order
    int* zrow;
    int* counts;    // out: [number of X pivots, number of Z pivots]
    int n, W;
};

// shared memory of one CTA holding R rows of W words
__host__ __device__ inline size_t sup_smem_bytes(int R, int W) { return (size_t)2 * R * (W | 1) * 8 + 16 + (size_t)3 * R; }

template <int WPL>  // words of a row per lane: W <= 32 * WPL
__global__ void __launch_bounds__(kSupThreads, 1) k_support_cluster(SupArgs A) {
    extern __shared__ __align__(16) uint64_t sup_sm[];
    const int C = cluster_nctarank(), rank = cluster_ctarank();
    const int n = A.n, W = A.W, S = W | 1;  // odd row stride: the lanes' reads of one word of 32 rows spread over the banks
    const int R = (n + C - 1) / C;
    const int RW = (R + kSupWarps - 1) / kSupWarps;
    uint64_t* lx = sup_sm;
    uint64_t* lz = lx + (size_t)R * S;
    int* lmin = (int*)(lz + (size_t)R * S);  // three rotating candidate slots
    uint8_t* lr = (uint8_t*)(lmin + 4);
    uint8_t* lu = lr + R;   // taken as an X pivot
    uint8_t* lzu = lu + R;  // taken as a Z pivot
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int r0 = rank * R;
    const int nloc = max(0, min(R, n - r0));
    for (int i = threadIdx.x; i < R * W; i += blockDim.x) {
        const int t = i / W, v = i - t * W;
        const bool in = t < nloc;
        lx[t * S + v] = in ? A.sx[(int64_t)(r0 + t) * W + v] : 0;
        lz[t * S + v] = in ? A.sz[(int64_t)(r0 + t) * W + v] : 0;
    }
    for (int t = threadIdx.x; t < R; t += blockDim.x) {
        lr[t] = t < nloc ? A.sr[r0 + t] : 0;
        lu[t] = 0;
        lzu[t] = 0;
    }
    if (threadIdx.x < 3) lmin[threadIdx.x] = INT_MAX;
    cluster_barrier();  // every CTA of the cluster running and initialised before the first remote read
    const int w0 = warp * RW, w1 = min(w0 + RW, nloc);
    const uint32_t slot_base = lane < C ? dsmem_map(lmin, lane) : 0u;
    int np = 0, nz = 0, k = 0;
    for (int phase = 0; phase < 2; ++phase) {
        uint64_t* M = phase == 0 ? lx : lz;
        for (int q = 0; q < n; ++q, ++k) {
            const int qw = q >> 6, slot = k % 3;
            const uint64_t qb = 1ull << (q & 63);
            for (int base = w0; base < w1; base += 32) {  // this warp's lowest eligible row
                const int t = base + lane;
                const bool hit = t < w1 && (M[t * S + qw] & qb) && !lu[t] && (phase == 0 || !lzu[t]);
                const unsigned m = __ballot_sync(0xffffffffu, hit);
                if (m) {
                    if (lane == 0) atomicMin(&lmin[slot], r0 + base + __ffs(m) - 1);
                    break;
                }
            }
            cluster_barrier();
            // the slot read two columns ago is free again: every CTA passed this barrier after reading it
            if (threadIdx.x == 0) lmin[(k + 2) % 3] = INT_MAX;
            const int p = __reduce_min_sync(0xffffffffu, lane < C ? dsmem_s32(slot_base + 4u * slot) : INT_MAX);
            if (p == INT_MAX) continue;  // no pivot for this column (the same answer in every CTA)
            const int owner = p / R, pl = p - owner * R;
            if (owner == rank && pl >= w0 && pl < w1 && lane == 0) {
                if (phase == 0) {
                    lu[pl] = 1;
                    A.pivots[np] = p;
                } else {
                    lzu[pl] = 1;
                    A.zcol[nz] = q;
                    A.zrow[nz] = p;
                }
            }
            if (phase == 0) ++np; else ++nz;
            uint64_t px[WPL], pz[WPL];
            const uint32_t ax = dsmem_map(lx + (size_t)pl * S, owner), az = dsmem_map(lz + (size_t)pl * S, owner);
#pragma unroll
            for (int j = 0; j < WPL; ++j) {
                const int v = lane + 32 * j;
                px[j] = (phase == 0 && v < W) ? dsmem_u64(ax + 8u * v) : 0;
                pz[j] = v < W ? dsmem_u64(az + 8u * v) : 0;
            }
            const int psign = dsmem_u8(dsmem_map(lr + pl, owner));
            for (int base = w0; base < w1; base += 32) {
                const int t = base + lane;
                const bool hit = t < w1 && r0 + t != p && (M[t * S + qw] & qb) && (phase == 0 || !lu[t]);
                unsigned m = __ballot_sync(0xffffffffu, hit);
                while (m) {
                    const int tt = base + __ffs(m) - 1;
                    m &= m - 1;
                    if (phase == 0) {
                        int g = 0;
#pragma unroll
                        for (int j = 0; j < WPL; ++j) {
                            const int v = lane + 32 * j;
                            if (v < W) {
                                const uint64_t x1 = px[j], z1 = pz[j], x2 = lx[tt * S + v], z2 = lz[tt * S + v];
                                const uint64_t plus = (x1 & z1 & ~x2 & z2) | (x1 & ~z1 & x2 & z2) | (~x1 & z1 & x2 & ~z2);
                                const uint64_t minus = (x1 & z1 & x2 & ~z2) | (x1 & ~z1 & ~x2 & z2) | (~x1 & z1 & x2 & z2);
                                g += __popcll(plus) - __popcll(minus);
                                lx[tt * S + v] = x2 ^ x1;
                                lz[tt * S + v] = z2 ^ z1;
                            }
                        }
                        g = __reduce_add_sync(0xffffffffu, g);
                        if (lane == 0) {
                            const int total = 2 * lr[tt] + 2 * psign + g;
                            lr[tt] = (((total % 4) + 4) % 4) == 2 ? 1 : 0;
                        }
                    } else {
#pragma unroll
                        for (int j = 0; j < WPL; ++j) {
                            const int v = lane + 32 * j;
                            if (v < W) lz[tt * S + v] ^= pz[j];
                        }
                        if (lane == 0) lr[tt] ^= (uint8_t)psign;
                    }
                }
            }
            __syncwarp();  // this warp's row and flag updates seen by all its lanes at the next column
        }
    }
    cluster_barrier();  // no CTA leaves while another may still read its rows
    for (int i = threadIdx.x; i < nloc * W; i += blockDim.x) {
        const int t = i / W, v = i - t * W;
        A.sx[(int64_t)(r0 + t) * W + v] = lx[t * S + v];
        A.sz[(int64_t)(r0 + t) * W + v] = lz[t * S + v];
    }
    for (int t = threadIdx.x; t < nloc; t += blockDim.x) {
        A.sr[r0 + t] = lr[t];
        A.used[r0 + t] = lu[t];
    }
    if (rank == 0 && threadIdx.x == 0) {
        A.counts[0] = np;
        A.counts[1] = nz;
    }
}

// cluster size for n rows, or 0 when this device cannot run the one-launch support
static int support_cluster_size(int n, int W, size_t* smem) {
    if (getenv("LSG_SUPPORT_STEPS")) return 0;  // diagnostics: the launch-per-column path
    int C = 1;
    while (C < kSupMaxCluster && (n + C - 1) / C > kSupRowsPerCta) C *= 2;
    const int R = (n + C - 1) / C;
    *smem = sup_smem_bytes(R, W);
    int dev = 0, optin = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess ||
        (size_t)optin < *smem || W > 64)
        return 0;
    auto kern = W <= 32 ? k_support_cluster<1> : k_support_cluster<2>;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)*smem) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = C;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(C);
    cfg.blockDim = dim3(kSupThreads);
    cfg.dynamicSmemBytes = *smem;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int clusters = 0;
    if (cudaOccupancyMaxActiveClusters(&clusters, kern, &cfg) != cudaSuccess || clusters < 1) {
        cudaGetLastError();
        return 0;
    }
    return C;
}

static cudaError_t launch_support_cluster(const SupArgs& A, int C, size_t smem, cudaStream_t st) {
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = C;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(C);
    cfg.blockDim = dim3(kSupThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return A.W <= 32 ? cudaLaunchKernelEx(&cfg, k_support_cluster<1>, A) : cudaLaunchKernelEx(&cfg, k_support_cluster<2>, A);
}

// Pauli frames: one CTA per 32-shot word.
struct FrameArgs {
    int n, shots;
    const GateRec* gates;
    const int64_t* moments;
    int64_t nmoments;
    const CTable* tables;
    const NTable* noise;
    const u128* gate_states;  // per noisy gate: the generator state before its block of uniforms
    u128 inc;
    u128 jmul, jplus;  // jump by 32 * blockIdx.x steps is computed per block from these per-word tables
    const u128* word_mult;
    const u128* word_plus;
    u128 s0;  // generator state at the start of the run (no uint32 buffered)
    const uint4* masks;  // the noise masks of k_noise_masks, or null: drawn here, per gate
    int64_t nnoisy;
    // outputs
    uint32_t* fx;  // n x words (the final X parts of the frames)
    int words;
};

__global__ void k_frames(FrameArgs A) {
    extern __shared__ uint32_t sm[];
    const int n = A.n;
    uint32_t* X = sm;
    uint32_t* Z = sm + n;
    const int w = blockIdx.x;
    const int shot0 = 32 * w;
    const int valid = min(32, A.shots - shot0);
    // initial frames: X = 0, Z = integers(0, 2, size=(n, shots), dtype=uint8): value (q, s) is
    // uint8 number q * shots + s of the stream
    for (int q = threadIdx.x; q < n; q += blockDim.x) {
        uint32_t zw = 0;
        const uint64_t base = (uint64_t)q * A.shots + shot0;
        uint64_t cur_raw_index = ~0ull;
        uint64_t raw = 0;
        for (int j = 0; j < valid; ++j) {
            const uint64_t t = base + j;
            const uint64_t ri = t >> 3;
            if (ri != cur_raw_index) {
                raw = pcg_raw(A.s0, A.inc, ri);
                cur_raw_index = ri;
            }
            const uint32_t word = ((t >> 2) & 1) ? (uint32_t)(raw >> 32) : (uint32_t)raw;
            zw |= (uint32_t)((word >> (8 * (t & 3) + 7)) & 1) << j;
        }
        X[q] = 0;
        Z[q] = zw;
    }
    __syncthreads();
    const u128 wm = A.word_mult[w], wp = A.word_plus[w];
    const u128 mult = pcg_mult();
    for (int64_t m = 0; m < A.nmoments; ++m) {
        const int64_t lo = A.moments[m], hi = A.moments[m + 1];
        for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
            const GateRec g = A.gates[i];
            frame_gate(X, Z, g, A.tables);
            if (g.noise < 0) continue;
            if (A.masks) {
                const uint4 mk = A.masks[(int64_t)w * A.nnoisy + g.nk];
                X[g.a] ^= mk.x;
                Z[g.a] ^= mk.y;
                if (mk.z | mk.w) {  // only two-qubit noise sets them
                    X[g.b] ^= mk.z;
                    Z[g.b] ^= mk.w;
                }
                continue;
            }
            const NTable& nt = A.noise[g.noise];
            // this word's shots draw uniforms number shot0 .. shot0+31 of the gate's block
            u128 st = wm * A.gate_states[g.nk] + wp;
            uint32_t mx[2] = {0, 0}, mz[2] = {0, 0};
            for (int j = 0; j < valid; ++j) {
                st = st * mult + A.inc;
                const uint64_t um = pcg_output(st) >> 11;  // the uniform is um * 2^-53
                int pick = 0;  // searchsorted(cumulative, u, side='right'), clamped
                while (pick < nt.nb && nt.thr[pick] <= um) ++pick;
                if (pick > nt.nb - 1) pick = nt.nb - 1;
                const uint8_t lab = nt.label[pick];
                for (int qi = 0; qi < nt.k; ++qi) {
                    const int sh = 2 * (nt.k - 1 - qi);
                    mx[qi] |= (uint32_t)((lab >> (sh + 1)) & 1) << j;
                    mz[qi] |= (uint32_t)((lab >> sh) & 1) << j;
                }
            }
            const int qs[2] = {g.a, g.b};
            for (int qi = 0; qi < nt.k; ++qi) {
                X[qs[qi]] ^= mx[qi];
                Z[qs[qi]] ^= mz[qi];
            }
        }
        __syncthreads();
    }
    for (int q = threadIdx.x; q < n; q += blockDim.x) A.fx[(int64_t)q * A.words + w] = X[q];
}

// outcome bits: bit (shot, pair) = x0[pos] ^ frame X of the qubit, then readout flips drawn at
// raw index flip_base + e * shots + shot for the e-th pair with an error (stabilizer.py:622-643)
__global__ void k_frames_out(const uint32_t* __restrict__ fx, int words, int shots, int npairs, const int* __restrict__ pq,
                             const int* __restrict__ pc, const int* __restrict__ perr, const double* __restrict__ p01,
                             const double* __restrict__ p10, const uint8_t* __restrict__ x0pos, u128 s0, u128 inc,
                             uint64_t flip_base, int nclbits, uint8_t* __restrict__ out) {
    const int64_t total = (int64_t)shots * npairs;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int s = (int)(t % shots), j = (int)(t / shots);
        const int q = pq[j];
        int v = ((fx ? (fx[(int64_t)q * words + (s >> 5)] >> (s & 31)) & 1 : 0)) ^ x0pos[j];
        if (perr[j] >= 0) {
            const double u = pcg_double(pcg_raw(s0, inc, flip_base + (uint64_t)perr[j] * shots + s));
            if (u < (v ? p10[j] : p01[j])) v ^= 1;
        }
        out[(int64_t)s * nclbits + pc[j]] = (uint8_t)v;
    }
}

// ideal sampling: outcome of shot s = x0 ^ XOR of basis rows i where integer (s * nb + i) is 1;
// one block per shot: the shot's coefficient bits first (one jump per raw draw), then the XORs
__global__ void k_sampled(const uint64_t* __restrict__ basis, int nb, int W, const uint64_t* __restrict__ x0, int shots,
                          u128 s0, u128 inc, uint64_t* __restrict__ outw) {
    __shared__ uint32_t coef[64];  // up to 2048 basis rows
    for (int s = blockIdx.x; s < shots; s += gridDim.x) {
        for (int i = threadIdx.x; i < 64; i += blockDim.x) coef[i] = 0;
        __syncthreads();
        const uint64_t t0 = (uint64_t)s * nb, t1 = t0 + nb;  // integers [t0, t1)
        const uint64_t r0 = t0 >> 3, r1 = (t1 + 7) >> 3;     // raw draws covering them
        for (uint64_t ri = r0 + threadIdx.x; ri < r1; ri += blockDim.x) {
            const uint64_t raw = pcg_raw(s0, inc, ri);
            for (int j = 0; j < 8; ++j) {
                const uint64_t t = 8 * ri + j;
                if (t < t0 || t >= t1) continue;
                const uint32_t word = (j >> 2) ? (uint32_t)(raw >> 32) : (uint32_t)raw;
                if ((word >> (8 * (j & 3) + 7)) & 1) atomicOr(&coef[(t - t0) >> 5], 1u << ((t - t0) & 31));
            }
        }
        __syncthreads();
        for (int v = threadIdx.x; v < W; v += blockDim.x) {
            uint64_t acc = x0[v];
            for (int i = 0; i < nb; ++i)
                if ((coef[i >> 5] >> (i & 31)) & 1) acc ^= basis[(int64_t)i * W + v];
            outw[(int64_t)s * W + v] = acc;
        }
        __syncthreads();
    }
}

__global__ void k_words_to_pairs(const uint64_t* __restrict__ outw, int W, int shots, int npairs, const int* __restrict__ ppos,
                                 const int* __restrict__ pc, const int* __restrict__ perr, const double* __restrict__ p01,
                                 const double* __restrict__ p10, u128 s0, u128 inc, uint64_t flip_base, int nclbits,
                                 uint8_t* __restrict__ out) {
    const int64_t total = (int64_t)shots * npairs;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int s = (int)(t % shots), j = (int)(t / shots);
        const int pos = ppos[j];
        int v = (int)((outw[(int64_t)s * W + (pos >> 6)] >> (pos & 63)) & 1);
        if (perr[j] >= 0) {
            const double u = pcg_double(pcg_raw(s0, inc, flip_base + (uint64_t)perr[j] * shots + s));
            if (u < (v ? p10[j] : p01[j])) v ^= 1;
        }
        out[(int64_t)s * nclbits + pc[j]] = (uint8_t)v;
    }
}

__global__ void k_gate_states(u128 s0, u128 inc, uint64_t base, uint64_t stride, int64_t count, u128* out) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < count; k += (int64_t)gridDim.x * blockDim.x)
        out[k] = pcg_advance(s0, inc, base + (uint64_t)k * stride);
}

// The Pauli-noise masks of every noisy gate for every 32-shot word, over all SMs: a warp per
// (gate, word), lane j drawing shot 32w + j's uniform (the gate's block state advanced by
// 32w + j + 1: word jump, then lane jump) and choosing its branch; ballots give the word's X and Z
// masks of the gate's (up to two) qubits. masks[w * nnoisy + nk] = {x0, z0, x1, z1}.
__global__ void k_noise_masks(const u128* __restrict__ gate_states, const int16_t* __restrict__ gate_table,
                              const NTable* __restrict__ noise, int64_t nnoisy, int words, int shots,
                              const u128* __restrict__ word_mult, const u128* __restrict__ word_plus,
                              const u128* __restrict__ lane_mult, const u128* __restrict__ lane_plus, uint4* masks) {
    const int lane = threadIdx.x & 31;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const u128 lm = lane_mult[lane], lp = lane_plus[lane];
    for (int64_t t = (((int64_t)blockIdx.x * blockDim.x) + threadIdx.x) >> 5; t < nnoisy * words; t += nwarps) {
        const int w = (int)(t / nnoisy);
        const int64_t nk = t - (int64_t)w * nnoisy;
        const NTable& nt = noise[gate_table[nk]];
        const u128 st = lm * (word_mult[w] * gate_states[nk] + word_plus[w]) + lp;
        const uint64_t m = pcg_output(st) >> 11;
        int pick = 0;  // searchsorted(cumulative, u, side='right'), clamped
        while (pick < nt.nb && nt.thr[pick] <= m) ++pick;
        if (pick > nt.nb - 1) pick = nt.nb - 1;
        const bool live = 32 * w + lane < shots;
        const unsigned lab = live ? nt.label[pick] : 0u;
        const int sh = 2 * (nt.k - 1);  // the first qubit's bits
        uint4 out;
        out.x = __ballot_sync(0xffffffffu, (lab >> (sh + 1)) & 1);
        out.y = __ballot_sync(0xffffffffu, (lab >> sh) & 1);
        out.z = nt.k == 2 ? __ballot_sync(0xffffffffu, (lab >> 1) & 1) : 0u;
        out.w = nt.k == 2 ? __ballot_sync(0xffffffffu, lab & 1) : 0u;
        if (lane == 0) masks[t] = out;
    }
}

// ASAP moments of a gate list: a gate's moment is one past the latest moment among its qubits
static void moments_of(const GateRec* g, int64_t ng, int n, const int8_t* arity, std::vector<int64_t>& order,
                       std::vector<int64_t>& starts) {
    std::vector<int64_t> last(n, -1), level(ng);
    int64_t maxl = -1;
    for (int64_t i = 0; i < ng; ++i) {
        int64_t l = last[g[i].a];
        if (arity[i] > 1) l = std::max(l, last[g[i].b]);
        if (arity[i] > 2) l = std::max(l, last[g[i].c]);
        level[i] = l + 1;
        last[g[i].a] = level[i];
        if (arity[i] > 1) last[g[i].b] = level[i];
        if (arity[i] > 2) last[g[i].c] = level[i];
        maxl = std::max(maxl, level[i]);
    }
    std::vector<int64_t> count(maxl + 2, 0);
    for (int64_t i = 0; i < ng; ++i) count[level[i] + 1]++;
    for (int64_t l = 0; l <= maxl; ++l) count[l + 1] += count[l];
    starts.assign(count.begin(), count.end());
    order.assign(ng, 0);
    std::vector<int64_t> fill(count.begin(), count.end() - 1);
    for (int64_t i = 0; i < ng; ++i) order[fill[level[i]]++] = i;
}

}  // namespace lsg

using namespace lsg;

struct lsg_tab_s {
    int n = 0, words = 0;  // words: 32-row words per qubit (2n rows)
    uint32_t *x = nullptr, *z = nullptr, *r = nullptr;
    cudaStream_t stream = nullptr;
    Scratch work, work2;
};

namespace {

int gate_records(int n, const lsg_cgate* gates, int64_t ng, int32_t ntables, int32_t nnoise, std::vector<GateRec>& recs,
                 std::vector<int8_t>& arity) {
    recs.resize(ng);
    arity.resize(ng);
    for (int64_t i = 0; i < ng; ++i) {
        const lsg_cgate& g = gates[i];
        int k = 1;
        if (g.code == 7 || g.code == 8) k = 2;
        else if (g.code >= 16) {
            if (g.code - 16 >= ntables) return fail(LSG_E_ARG, "gate %lld names a missing table", (long long)i);
            k = g.nq;
            if (k < 1 || k > 3) return fail(LSG_E_ARG, "gate %lld has a bad arity", (long long)i);
        } else if (g.code < 0 || g.code > 8) {
            return fail(LSG_E_ARG, "gate %lld has a bad code", (long long)i);
        }
        const int q[3] = {g.a, g.b, g.c};
        for (int j = 0; j < k; ++j)
            if (q[j] < 0 || q[j] >= n) return fail(LSG_E_ARG, "gate %lld names a missing qubit", (long long)i);
        if (g.noise >= nnoise) return fail(LSG_E_ARG, "gate %lld names a missing noise table", (long long)i);
        recs[i] = GateRec{(int16_t)g.code, (int16_t)g.noise, (int16_t)g.a, (int16_t)g.b, (int16_t)g.c, 0, -1};
        arity[i] = (int8_t)k;
    }
    return LSG_OK;
}

int upload(Scratch& s, const void* host, size_t bytes, cudaStream_t st) {
    LSG_CHECK(ensure(s, bytes));
    if (bytes) LSG_CUDA(cudaMemcpyAsync(s.ptr, host, bytes, cudaMemcpyHostToDevice, st));
    return LSG_OK;
}

int tables_device(const uint8_t* tables, int32_t ntables, std::vector<CTable>& out) {
    out.resize(std::max(ntables, 1));
    for (int i = 0; i < ntables; ++i) {
        std::memset(&out[i], 0, sizeof(CTable));
        out[i].k = tables[i * 65];
        if (out[i].k < 1 || out[i].k > 3) return fail(LSG_E_ARG, "Clifford table %d has a bad width", i);
        std::memcpy(out[i].e, tables + i * 65 + 1, 64);
    }
    return LSG_OK;
}

}  // namespace

extern "C" {

int lsg_pcg_raw(const uint64_t* state, uint64_t index, uint64_t* out) {
    clear_error();
    if (!state || !out) return fail(LSG_E_ARG, "null argument");
    const u128 s = ((u128)state[0] << 64) | state[1];
    const u128 inc = ((u128)state[2] << 64) | state[3];
    *out = pcg_raw(s, inc, index);
    return LSG_OK;
}

int lsg_cgates_from_kinds(int64_t n, const int64_t* kind, int32_t nkinds, const int16_t* kind_code,
                          const int16_t* kind_nq, const int16_t* kind_noise, const int64_t* qubits, const int64_t* arity,
                          lsg_cgate* out) {
    clear_error();
    if (n < 0 || nkinds < 0 ||
        (n > 0 && (!kind || !kind_code || !kind_nq || !kind_noise || !qubits || !arity || !out)))
        return fail(LSG_E_ARG, "lsg_cgates_from_kinds: bad arguments");
    for (int64_t i = 0; i < n; ++i) {
        const int64_t k = kind[i], a = arity[i];
        if (k < 0 || k >= nkinds || a < 1 || a > 3)
            return fail(LSG_E_ARG, "lsg_cgates_from_kinds: gate %lld has kind %lld and %lld qubits", (long long)i,
                        (long long)k, (long long)a);
        int16_t q[3] = {0, 0, 0};
        for (int64_t j = 0; j < a; ++j) {
            const int64_t v = qubits[3 * i + j];
            if (v < 0 || v > 32767)
                return fail(LSG_E_ARG, "lsg_cgates_from_kinds: gate %lld names qubit %lld", (long long)i, (long long)v);
            q[j] = (int16_t)v;
        }
        lsg_cgate g;
        g.code = kind_code[k];
        g.noise = kind_noise[k];
        g.a = q[0];
        g.b = q[1];
        g.c = q[2];
        g.nq = kind_nq[k];
        g.pad = 0;
        out[i] = g;
    }
    return LSG_OK;
}

int lsg_tab_create(int n, lsg_tab* out) {
    clear_error();
    if (!out) return fail(LSG_E_ARG, "null output");
    *out = nullptr;
    if (n < 1 || n > 2048) return fail(LSG_E_CAPACITY, "%d qubits are more than the stabilizer engine allows (up to 2048)", n);
    auto* t = new lsg_tab_s();
    t->n = n;
    t->words = (2 * n + 31) / 32;
    const size_t bytes = (size_t)n * t->words * 4;
    if (cudaStreamCreateWithFlags(&t->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&t->x, bytes) != cudaSuccess || cudaMalloc(&t->z, bytes) != cudaSuccess ||
        cudaMalloc(&t->r, (size_t)t->words * 4) != cudaSuccess) {
        cudaGetLastError();
        lsg_tab_free(t);
        return fail(LSG_E_MEMORY, "cannot allocate the tableau");
    }
    // destabilizer i = X_i (row i), stabilizer i = Z_i (row n + i)
    std::vector<uint32_t> hx((size_t)n * t->words, 0), hz((size_t)n * t->words, 0);
    for (int i = 0; i < n; ++i) {
        hx[(size_t)i * t->words + (i >> 5)] |= 1u << (i & 31);
        const int row = n + i;
        hz[(size_t)i * t->words + (row >> 5)] |= 1u << (row & 31);
    }
    LSG_CUDA(cudaMemcpy(t->x, hx.data(), bytes, cudaMemcpyHostToDevice));
    LSG_CUDA(cudaMemcpy(t->z, hz.data(), bytes, cudaMemcpyHostToDevice));
    LSG_CUDA(cudaMemset(t->r, 0, (size_t)t->words * 4));
    *out = t;
    return LSG_OK;
}

int lsg_tab_free(lsg_tab t) {
    clear_error();
    if (!t) return LSG_OK;
    if (t->stream) cudaStreamSynchronize(t->stream);
    cudaFree(t->x);
    cudaFree(t->z);
    cudaFree(t->r);
    release(t->work);
    release(t->work2);
    if (t->stream) cudaStreamDestroy(t->stream);
    delete t;
    return LSG_OK;
}

int lsg_tab_apply(lsg_tab t, const lsg_cgate* gates, int64_t ngates, const uint8_t* tables, int32_t ntables) {
    clear_error();
    if (!t || ngates < 0 || (ngates && !gates) || ntables < 0 || (ntables && !tables)) return fail(LSG_E_ARG, "bad arguments");
    if (ngates == 0) return LSG_OK;
    std::vector<GateRec> recs;
    std::vector<int8_t> arity;
    LSG_CHECK(gate_records(t->n, gates, ngates, ntables, 0x7fff, recs, arity));
    std::vector<int64_t> order, starts;
    moments_of(recs.data(), ngates, t->n, arity.data(), order, starts);
    std::vector<GateRec> sorted(ngates);
    for (int64_t i = 0; i < ngates; ++i) sorted[i] = recs[order[i]];
    std::vector<CTable> ct;
    LSG_CHECK(tables_device(tables, ntables, ct));
    const size_t gb = ngates * sizeof(GateRec), mb = starts.size() * 8, tb = ct.size() * sizeof(CTable);
    const size_t o_m = (gb + 255) & ~size_t(255), o_t = o_m + ((mb + 255) & ~size_t(255));
    LSG_CHECK(ensure(t->work, o_t + tb));
    char* base = (char*)t->work.ptr;
    LSG_CUDA(cudaMemcpyAsync(base, sorted.data(), gb, cudaMemcpyHostToDevice, t->stream));
    LSG_CUDA(cudaMemcpyAsync(base + o_m, starts.data(), mb, cudaMemcpyHostToDevice, t->stream));
    LSG_CUDA(cudaMemcpyAsync(base + o_t, ct.data(), tb, cudaMemcpyHostToDevice, t->stream));
    const size_t smem = (size_t)2 * t->n * 4;
    k_tab_apply<<<t->words, kS, smem, t->stream>>>(t->x, t->z, t->r, t->n, t->words, (const GateRec*)base,
                                                   (const int64_t*)(base + o_m), (int64_t)starts.size() - 1,
                                                   (const CTable*)(base + o_t));
    LSG_CUDA(cudaGetLastError());
    LSG_CUDA(cudaStreamSynchronize(t->stream));
    return LSG_OK;
}

int lsg_tab_download(lsg_tab t, uint8_t* x, uint8_t* z, uint8_t* r) {
    clear_error();
    if (!t || !x || !z || !r) return fail(LSG_E_ARG, "null argument");
    const int n = t->n, W = t->words;
    std::vector<uint32_t> hx((size_t)n * W), hz((size_t)n * W), hr(W);
    LSG_CUDA(cudaMemcpyAsync(hx.data(), t->x, hx.size() * 4, cudaMemcpyDeviceToHost, t->stream));
    LSG_CUDA(cudaMemcpyAsync(hz.data(), t->z, hz.size() * 4, cudaMemcpyDeviceToHost, t->stream));
    LSG_CUDA(cudaMemcpyAsync(hr.data(), t->r, hr.size() * 4, cudaMemcpyDeviceToHost, t->stream));
    LSG_CUDA(cudaStreamSynchronize(t->stream));
    for (int q = 0; q < n; ++q)
        for (int row = 0; row < 2 * n; ++row) {
            x[(size_t)q * 2 * n + row] = (hx[(size_t)q * W + (row >> 5)] >> (row & 31)) & 1;
            z[(size_t)q * 2 * n + row] = (hz[(size_t)q * W + (row >> 5)] >> (row & 31)) & 1;
        }
    for (int row = 0; row < 2 * n; ++row) r[row] = (hr[row >> 5] >> (row & 31)) & 1;
    return LSG_OK;
}

// support() with a launch per column and phase (the path for devices that cannot run the
// one-launch cluster kernel): pivot kernels and rowsum/XOR kernels, the Z constraints compacted
// on the host
static int support_steps(int n, int W, uint64_t* sx, uint64_t* sz, uint8_t* sr, char* b, size_t o_used, size_t o_piv, size_t o_pivots, size_t o_np, size_t o_zm,
                         size_t o_zb, size_t o_zp, size_t o_znp, size_t o_zused, cudaStream_t st,
                         std::vector<uint8_t>& xfull, std::vector<int>& pivots, std::vector<uint64_t>& hsx) {
    const size_t rowsb = (size_t)n * W * 8;
    LSG_CUDA(cudaMemsetAsync(b + o_used, 0, n, st));
    LSG_CUDA(cudaMemsetAsync(b + o_np, 0, 8, st));
    const unsigned rg = (unsigned)std::max(1, std::min(152 * 4, (n * 32 + kS - 1) / kS));
    for (int q = 0; q < n; ++q) {
        k_elim_pivot<<<1, 1024, 0, st>>>(sx, n, W, q, (uint8_t*)(b + o_used), (int*)(b + o_piv), (int*)(b + o_pivots),
                                        (int*)(b + o_np), 1);
        k_sup_rowsum<<<rg, kS, 0, st>>>(sx, sz, sr, n, W, q, (const int*)(b + o_piv));
    }
    LSG_CUDA(cudaGetLastError());
    // Z constraints of the unused rows, in row order (stabilizer.py:359-360, :398-422)
    std::vector<uint8_t> used(n);
    int npiv = 0;
    LSG_CUDA(cudaMemcpyAsync(used.data(), b + o_used, n, cudaMemcpyDeviceToHost, st));
    LSG_CUDA(cudaMemcpyAsync(&npiv, b + o_np, 4, cudaMemcpyDeviceToHost, st));
    LSG_CUDA(cudaStreamSynchronize(st));
    pivots.assign(npiv, 0);
    if (npiv) LSG_CUDA(cudaMemcpy(pivots.data(), b + o_pivots, (size_t)npiv * 4, cudaMemcpyDeviceToHost));
    std::vector<uint64_t> hsz((size_t)n * W);
    std::vector<uint8_t> hsr(n);
    LSG_CUDA(cudaMemcpy(hsz.data(), sz, rowsb, cudaMemcpyDeviceToHost));
    LSG_CUDA(cudaMemcpy(hsx.data(), sx, rowsb, cudaMemcpyDeviceToHost));
    LSG_CUDA(cudaMemcpy(hsr.data(), sr, n, cudaMemcpyDeviceToHost));
    std::vector<uint64_t> zm;
    std::vector<uint8_t> zb;
    for (int i = 0; i < n; ++i)
        if (!used[i]) {
            zm.insert(zm.end(), hsz.begin() + (size_t)i * W, hsz.begin() + (size_t)(i + 1) * W);
            zb.push_back(hsr[i]);
        }
    const int zr = (int)zb.size();
    if (zr == 0) return LSG_OK;
    LSG_CUDA(cudaMemcpyAsync(b + o_zm, zm.data(), zm.size() * 8, cudaMemcpyHostToDevice, st));
    LSG_CUDA(cudaMemcpyAsync(b + o_zb, zb.data(), zr, cudaMemcpyHostToDevice, st));
    LSG_CUDA(cudaMemsetAsync(b + o_zused, 0, zr, st));
    LSG_CUDA(cudaMemsetAsync(b + o_znp, 0, 8, st));
    const unsigned zg = (unsigned)std::max(1, std::min(152 * 4, (zr * 32 + kS - 1) / kS));
    for (int q = 0; q < n; ++q) {
        k_elim_pivot<<<1, 1024, 0, st>>>((uint64_t*)(b + o_zm), zr, W, q, (uint8_t*)(b + o_zused), (int*)(b + o_piv),
                                        (int*)(b + o_zp), (int*)(b + o_znp), 1);
        k_elim_xor<<<zg, kS, 0, st>>>((uint64_t*)(b + o_zm), (uint8_t*)(b + o_zb), zr, W, q, (const int*)(b + o_piv));
    }
    LSG_CUDA(cudaGetLastError());
    int nz = 0;
    LSG_CUDA(cudaMemcpyAsync(&nz, b + o_znp, 4, cudaMemcpyDeviceToHost, st));
    LSG_CUDA(cudaStreamSynchronize(st));
    std::vector<int> zp(nz);
    std::vector<uint8_t> fb(zr);
    std::vector<uint64_t> fm((size_t)zr * W);
    if (nz) LSG_CUDA(cudaMemcpy(zp.data(), b + o_zp, (size_t)nz * 4, cudaMemcpyDeviceToHost));
    LSG_CUDA(cudaMemcpy(fb.data(), b + o_zb, zr, cudaMemcpyDeviceToHost));
    LSG_CUDA(cudaMemcpy(fm.data(), b + o_zm, (size_t)zr * W * 8, cudaMemcpyDeviceToHost));
    // pivots are taken for ascending columns and the reduction is full, so the column of a
    // pivot row is its lowest set bit: no earlier column survives in it
    for (int j = 0; j < nz; ++j) {
        const int p = zp[j];
        int col = -1;
        for (int v = 0; v < W && col < 0; ++v)
            if (fm[(size_t)p * W + v]) col = 64 * v + __builtin_ctzll(fm[(size_t)p * W + v]);
        if (col >= 0 && col < n) xfull[col] = fb[p];
    }
    return LSG_OK;
}

int lsg_tab_support(lsg_tab t, const int32_t* qubits, int32_t m, uint8_t* x0, uint8_t* basis, int32_t* rank) {
    clear_error();
    if (!t || !qubits || !x0 || m < 1 || !rank) return fail(LSG_E_ARG, "bad arguments");
    const int n = t->n;
    for (int i = 0; i < m; ++i)
        if (qubits[i] < 0 || qubits[i] >= n) return fail(LSG_E_ARG, "support: qubit out of range");
    const int W = (n + 63) / 64;
    cudaStream_t st = t->stream;
    // device work: sx | sz | sr | used | pivot | pivots | npiv | solve buffers
    auto al = [](size_t v) { return (v + 255) & ~size_t(255); };
    const size_t rowsb = (size_t)n * W * 8;
    size_t off = 0;
    const size_t o_sx = off; off += al(rowsb);
    const size_t o_sz = off; off += al(rowsb);
    const size_t o_sr = off; off += al(n);
    const size_t o_used = off; off += al(n);
    const size_t o_piv = off; off += al(8);
    const size_t o_pivots = off; off += al((size_t)n * 4);
    const size_t o_np = off; off += al(8);
    const size_t o_zm = off; off += al(rowsb);
    const size_t o_zb = off; off += al(n);
    const size_t o_zp = off; off += al((size_t)n * 4);
    const size_t o_znp = off; off += al(8);
    const size_t o_zused = off; off += al(n);
    const size_t o_zc = off; off += al((size_t)n * 4);
    const size_t o_zrw = off; off += al((size_t)n * 4);
    LSG_CHECK(ensure(t->work2, off));
    char* b = (char*)t->work2.ptr;
    uint64_t* sx = (uint64_t*)(b + o_sx);
    uint64_t* sz = (uint64_t*)(b + o_sz);
    uint8_t* sr = (uint8_t*)(b + o_sr);
    k_tab_rows<<<std::max(1, std::min(152 * 8, (n * W + kS - 1) / kS)), kS, 0, st>>>(t->x, t->z, t->r, n, t->words, W, sx,
                                                                                   sz, sr);
    std::vector<uint8_t> xfull(n, 0);
    std::vector<int> pivots;
    std::vector<uint64_t> hsx((size_t)n * W);
    size_t smem = 0;
    const int C = support_cluster_size(n, W, &smem);
    if (C > 0) {
        SupArgs A;
        A.sx = sx;
        A.sz = sz;
        A.sr = sr;
        A.used = (uint8_t*)(b + o_used);
        A.pivots = (int*)(b + o_pivots);
        A.zcol = (int*)(b + o_zc);
        A.zrow = (int*)(b + o_zrw);
        A.counts = (int*)(b + o_np);
        A.n = n;
        A.W = W;
        LSG_CUDA(launch_support_cluster(A, C, smem, st));
        int counts[2] = {0, 0};
        LSG_CUDA(cudaMemcpyAsync(counts, A.counts, 8, cudaMemcpyDeviceToHost, st));
        LSG_CUDA(cudaStreamSynchronize(st));
        const int npiv = counts[0], nz = counts[1];
        if (npiv < 0 || npiv > n || nz < 0 || nz > n) return fail(LSG_E_CUDA, "support: bad pivot counts %d, %d", npiv, nz);
        pivots.resize(npiv);
        std::vector<int> zc(nz), zrw(nz);
        std::vector<uint8_t> hsr(n);
        if (npiv) LSG_CUDA(cudaMemcpyAsync(pivots.data(), A.pivots, (size_t)npiv * 4, cudaMemcpyDeviceToHost, st));
        if (nz) {
            LSG_CUDA(cudaMemcpyAsync(zc.data(), A.zcol, (size_t)nz * 4, cudaMemcpyDeviceToHost, st));
            LSG_CUDA(cudaMemcpyAsync(zrw.data(), A.zrow, (size_t)nz * 4, cudaMemcpyDeviceToHost, st));
        }
        LSG_CUDA(cudaMemcpyAsync(hsr.data(), sr, n, cudaMemcpyDeviceToHost, st));
        LSG_CUDA(cudaMemcpyAsync(hsx.data(), sx, rowsb, cudaMemcpyDeviceToHost, st));
        LSG_CUDA(cudaStreamSynchronize(st));
        // the solution of the Z constraints: each pivot column takes its reduced row's sign
        for (int j = 0; j < nz; ++j) {
            if (zc[j] < 0 || zc[j] >= n || zrw[j] < 0 || zrw[j] >= n) return fail(LSG_E_CUDA, "support: bad Z pivot %d", j);
            xfull[zc[j]] = hsr[zrw[j]];
        }
        for (int j = 0; j < npiv; ++j)
            if (pivots[j] < 0 || pivots[j] >= n) return fail(LSG_E_CUDA, "support: bad X pivot %d", j);
    } else {
        LSG_CHECK(support_steps(n, W, sx, sz, sr, b, o_used, o_piv, o_pivots, o_np, o_zm, o_zb, o_zp, o_znp, o_zused, st, xfull,
                                pivots, hsx));
    }
    const int npiv = (int)pivots.size();
    for (int i = 0; i < m; ++i) x0[i] = xfull[qubits[i]];
    // basis: X parts of the pivot rows restricted to `qubits` (stabilizer.py:361-365)
    bool identity = m == n;
    for (int i = 0; identity && i < m; ++i) identity = qubits[i] == i;
    std::vector<uint8_t> vec((size_t)npiv * m);
    for (int j = 0; j < npiv; ++j)
        for (int i = 0; i < m; ++i) {
            const int q = qubits[i];
            vec[(size_t)j * m + i] = (hsx[(size_t)pivots[j] * W + (q >> 6)] >> (q & 63)) & 1;
        }
    if (identity) {
        *rank = npiv;
        if (basis) std::memcpy(basis, vec.data(), vec.size());
        return LSG_OK;
    }
    // row basis of the restricted vectors (stabilizer.py:425-440), on the host: npiv x m bits
    const int Wm = (m + 63) / 64;
    std::vector<uint64_t> mm((size_t)npiv * Wm, 0);
    for (int j = 0; j < npiv; ++j)
        for (int i = 0; i < m; ++i)
            if (vec[(size_t)j * m + i]) mm[(size_t)j * Wm + (i >> 6)] |= 1ull << (i & 63);
    std::vector<uint64_t> out;
    int nb = 0;
    for (int col = 0; col < m && nb < m; ++col) {
        int p = -1;
        for (int j = 0; j < npiv; ++j)
            if ((mm[(size_t)j * Wm + (col >> 6)] >> (col & 63)) & 1) {
                p = j;
                break;
            }
        if (p < 0) continue;
        std::vector<uint64_t> row(mm.begin() + (size_t)p * Wm, mm.begin() + (size_t)(p + 1) * Wm);
        out.insert(out.end(), row.begin(), row.end());
        ++nb;
        for (int j = 0; j < npiv; ++j)
            if ((mm[(size_t)j * Wm + (col >> 6)] >> (col & 63)) & 1)
                for (int v = 0; v < Wm; ++v) mm[(size_t)j * Wm + v] ^= row[v];
    }
    *rank = nb;
    if (basis)
        for (int j = 0; j < nb; ++j)
            for (int i = 0; i < m; ++i) basis[(size_t)j * m + i] = (out[(size_t)j * Wm + (i >> 6)] >> (i & 63)) & 1;
    return LSG_OK;
}

int lsg_frames_run(int n, const lsg_cgate* gates, int64_t ngates, const uint8_t* tables, int32_t ntables,
                   const lsg_noise_table* noise, int32_t nnoise, int64_t shots, const uint64_t* rng_state,
                   int32_t npairs, const int32_t* pair_qubit, const int32_t* pair_clbit, const uint8_t* pair_x0,
                   const int32_t* pair_err, const double* p01, const double* p10, int32_t nclbits, uint8_t* bits_out,
                   int64_t* raw_used) {
    clear_error();
    if (n < 1 || n > 2048 || ngates < 0 || (ngates && !gates) || shots < 1 || !rng_state || npairs < 1 || !pair_qubit ||
        !pair_clbit || !pair_x0 || !pair_err || !p01 || !p10 || !bits_out || nclbits < 1 || nnoise < 0 ||
        (nnoise && !noise))
        return fail(LSG_E_ARG, "lsg_frames_run: bad arguments");
    if (shots > (1ll << 30)) return fail(LSG_E_ARG, "too many shots for one frames run");
    std::vector<GateRec> recs;
    std::vector<int8_t> arity;
    LSG_CHECK(gate_records(n, gates, ngates, ntables, nnoise, recs, arity));
    int64_t nk = 0;
    for (int64_t i = 0; i < ngates; ++i)
        if (recs[i].noise >= 0) recs[i].nk = (int32_t)nk++;
    for (int j = 0; j < npairs; ++j)
        if (pair_qubit[j] < 0 || pair_qubit[j] >= n || pair_clbit[j] < 0 || pair_clbit[j] >= nclbits)
            return fail(LSG_E_ARG, "lsg_frames_run: bad measurement pair %d", j);
    std::vector<NTable> nt(std::max(nnoise, 1));
    for (int i = 0; i < nnoise; ++i) {
        const lsg_noise_table& s = noise[i];
        if (s.k < 1 || s.k > 2 || s.nbranch < 1 || s.nbranch > 16) return fail(LSG_E_ARG, "noise table %d is malformed", i);
        nt[i].k = s.k;
        nt[i].nb = s.nbranch;
        for (int j = 0; j < 16; ++j) {
            nt[i].cum[j] = s.cumulative[j];
            nt[i].label[j] = s.label[j];
            const double c = s.cumulative[j];
            // exact: scaling by 2^53 and ceil are exact in FP64; c >= 1 is never <= a uniform
            nt[i].thr[j] = !(c > 0.0) ? 0ull : c >= 1.0 ? (1ull << 53) : (uint64_t)std::ceil(std::ldexp(c, 53));
        }
    }
    std::vector<int64_t> order, starts;
    moments_of(recs.data(), ngates, n, arity.data(), order, starts);
    std::vector<GateRec> sorted(ngates);
    for (int64_t i = 0; i < ngates; ++i) sorted[i] = recs[order[i]];
    std::vector<CTable> ct;
    LSG_CHECK(tables_device(tables, ntables, ct));
    const u128 s0 = ((u128)rng_state[0] << 64) | rng_state[1];
    const u128 inc = ((u128)rng_state[2] << 64) | rng_state[3];
    // draw layout: the frame bits (n * shots uint8 = ceil(n*shots/8) raw draws), then shots
    // uniforms per noisy gate in circuit order, then shots uniforms per readout pair with an error
    const uint64_t n8 = (uint64_t)n * shots;
    const uint64_t n32 = (n8 + 3) / 4;
    const uint64_t base_noise = (n32 + 1) / 2;
    const uint64_t base_flip = base_noise + (uint64_t)nk * shots;
    int nerr = 0;
    for (int j = 0; j < npairs; ++j)
        if (pair_err[j] >= 0) ++nerr;
    if (raw_used) *raw_used = (int64_t)(base_flip + (uint64_t)nerr * shots);
    const int words = (int)((shots + 31) / 32);
    std::vector<u128> wmul(words), wplus(words), lmul(32), lplus(32);
    for (int w = 0; w < words; ++w) pcg_jump(inc, (uint64_t)32 * w, &wmul[w], &wplus[w]);
    for (int j = 0; j < 32; ++j) pcg_jump(inc, (uint64_t)j + 1, &lmul[j], &lplus[j]);
    // the noise masks of all noisy gates and words drawn up front over every SM, when they fit a
    // quarter of the free device memory (else the frame kernel draws them per gate)
    std::vector<int16_t> gate_table((size_t)std::max<int64_t>(nk, 1), 0);
    for (int64_t i = 0; i < ngates; ++i)
        if (recs[i].noise >= 0) gate_table[(size_t)recs[i].nk] = recs[i].noise;
    const size_t mask_bytes = (size_t)nk * (size_t)words * sizeof(uint4);
    size_t free_mem = 0, total_mem = 0;
    const bool premask = nk > 0 && cudaMemGetInfo(&free_mem, &total_mem) == cudaSuccess && mask_bytes <= free_mem / 4;
    cudaStream_t st = nullptr;
    LSG_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    auto al = [](size_t v) { return (v + 255) & ~size_t(255); };
    size_t off = 0;
    const size_t o_g = off; off += al(ngates * sizeof(GateRec));
    const size_t o_m = off; off += al(starts.size() * 8);
    const size_t o_t = off; off += al(ct.size() * sizeof(CTable));
    const size_t o_n = off; off += al(nt.size() * sizeof(NTable));
    const size_t o_s = off; off += al((size_t)std::max<int64_t>(nk, 1) * 16);
    const size_t o_wm = off; off += al((size_t)words * 16);
    const size_t o_wp = off; off += al((size_t)words * 16);
    const size_t o_fx = off; off += al((size_t)n * words * 4);
    const size_t o_pq = off; off += al((size_t)npairs * 4);
    const size_t o_pc = off; off += al((size_t)npairs * 4);
    const size_t o_pe = off; off += al((size_t)npairs * 4);
    const size_t o_p0 = off; off += al((size_t)npairs * 8);
    const size_t o_p1 = off; off += al((size_t)npairs * 8);
    const size_t o_x0 = off; off += al((size_t)npairs);
    const size_t o_out = off; off += al((size_t)shots * nclbits);
    const size_t o_lm = off; off += al(32 * 16);
    const size_t o_lp = off; off += al(32 * 16);
    const size_t o_gt = off; off += al(gate_table.size() * sizeof(int16_t));
    const size_t o_mk = off; off += premask ? al(mask_bytes) : 0;
    Scratch work;
    int rc = ensure(work, off);
    if (rc != LSG_OK) {
        cudaStreamDestroy(st);
        return rc;
    }
    char* b = (char*)work.ptr;
    std::vector<int32_t> perr(npairs);
    {
        int e = 0;
        for (int j = 0; j < npairs; ++j) perr[j] = pair_err[j] >= 0 ? e++ : -1;
    }
    cudaError_t ce = cudaSuccess;
    auto H2D = [&](size_t o, const void* src, size_t bytes) {
        if (bytes && ce == cudaSuccess) ce = cudaMemcpyAsync(b + o, src, bytes, cudaMemcpyHostToDevice, st);
    };
    H2D(o_g, sorted.data(), ngates * sizeof(GateRec));
    H2D(o_m, starts.data(), starts.size() * 8);
    H2D(o_t, ct.data(), ct.size() * sizeof(CTable));
    H2D(o_n, nt.data(), nt.size() * sizeof(NTable));
    H2D(o_wm, wmul.data(), (size_t)words * 16);
    H2D(o_wp, wplus.data(), (size_t)words * 16);
    H2D(o_pq, pair_qubit, (size_t)npairs * 4);
    H2D(o_pc, pair_clbit, (size_t)npairs * 4);
    H2D(o_pe, perr.data(), (size_t)npairs * 4);
    H2D(o_p0, p01, (size_t)npairs * 8);
    H2D(o_p1, p10, (size_t)npairs * 8);
    H2D(o_x0, pair_x0, (size_t)npairs);
    H2D(o_lm, lmul.data(), 32 * 16);
    H2D(o_lp, lplus.data(), 32 * 16);
    if (premask) H2D(o_gt, gate_table.data(), gate_table.size() * sizeof(int16_t));
    if (ce == cudaSuccess) ce = cudaMemsetAsync(b + o_out, 0, (size_t)shots * nclbits, st);
    if (ce == cudaSuccess && nk)
        k_gate_states<<<std::max<int64_t>(1, std::min<int64_t>((nk + kS - 1) / kS, 152 * 64)), kS, 0, st>>>(
            s0, inc, base_noise, (uint64_t)shots, nk, (u128*)(b + o_s));
    FrameArgs A{};
    A.n = n;
    A.shots = (int)shots;
    A.gates = (const GateRec*)(b + o_g);
    A.moments = (const int64_t*)(b + o_m);
    A.nmoments = (int64_t)starts.size() - 1;
    A.tables = (const CTable*)(b + o_t);
    A.noise = (const NTable*)(b + o_n);
    A.gate_states = (const u128*)(b + o_s);
    A.inc = inc;
    A.word_mult = (const u128*)(b + o_wm);
    A.word_plus = (const u128*)(b + o_wp);
    A.s0 = s0;
    A.fx = (uint32_t*)(b + o_fx);
    A.words = words;
    A.masks = premask ? (const uint4*)(b + o_mk) : nullptr;
    A.nnoisy = nk;
    if (ce == cudaSuccess && premask) {
        const int64_t warps = nk * (int64_t)words;
        k_noise_masks<<<(unsigned)std::max<int64_t>(1, std::min<int64_t>((warps * 32 + kS - 1) / kS, 152 * 32)), kS, 0, st>>>(
            (const u128*)(b + o_s), (const int16_t*)(b + o_gt), (const NTable*)(b + o_n), nk, words, (int)shots,
            (const u128*)(b + o_wm), (const u128*)(b + o_wp), (const u128*)(b + o_lm), (const u128*)(b + o_lp),
            (uint4*)(b + o_mk));
        ce = cudaGetLastError();
    }
    if (ce == cudaSuccess) {
        k_frames<<<words, kS, (size_t)2 * n * 4, st>>>(A);
        ce = cudaGetLastError();
    }
    if (ce == cudaSuccess) {
        const int64_t tot = shots * npairs;
        k_frames_out<<<(unsigned)std::max<int64_t>(1, std::min<int64_t>((tot + kS - 1) / kS, 152 * 64)), kS, 0, st>>>(
            (const uint32_t*)(b + o_fx), words, (int)shots, npairs, (const int*)(b + o_pq), (const int*)(b + o_pc),
            (const int*)(b + o_pe), (const double*)(b + o_p0), (const double*)(b + o_p1), (const uint8_t*)(b + o_x0), s0,
            inc, base_flip, nclbits, (uint8_t*)(b + o_out));
        ce = cudaGetLastError();
    }
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(bits_out, b + o_out, (size_t)shots * nclbits, cudaMemcpyDeviceToHost, st);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
    release(work);
    cudaStreamDestroy(st);
    if (ce != cudaSuccess) return fail(LSG_E_CUDA, "the frames run failed: %s", cudaGetErrorString(ce));
    return LSG_OK;
}

int lsg_stab_sample(int m, const uint8_t* x0, const uint8_t* basis, int32_t nb, int64_t shots, const uint64_t* rng_state,
                    int32_t npairs, const int32_t* pair_pos, const int32_t* pair_clbit, const int32_t* pair_err,
                    const double* p01, const double* p10, int32_t nclbits, uint8_t* bits_out, int64_t* raw_used) {
    clear_error();
    if (m < 1 || !x0 || nb < 0 || (nb && !basis) || shots < 1 || !rng_state || npairs < 1 || !pair_pos || !pair_clbit ||
        !pair_err || !p01 || !p10 || nclbits < 1 || !bits_out)
        return fail(LSG_E_ARG, "lsg_stab_sample: bad arguments");
    for (int j = 0; j < npairs; ++j)
        if (pair_pos[j] < 0 || pair_pos[j] >= m || pair_clbit[j] < 0 || pair_clbit[j] >= nclbits)
            return fail(LSG_E_ARG, "lsg_stab_sample: bad pair %d", j);
    const int W = (m + 63) / 64;
    std::vector<uint64_t> bx((size_t)std::max(nb, 1) * W, 0), xw(W, 0);
    for (int i = 0; i < m; ++i)
        if (x0[i]) xw[i >> 6] |= 1ull << (i & 63);
    for (int j = 0; j < nb; ++j)
        for (int i = 0; i < m; ++i)
            if (basis[(size_t)j * m + i]) bx[(size_t)j * W + (i >> 6)] |= 1ull << (i & 63);
    const u128 s0 = ((u128)rng_state[0] << 64) | rng_state[1];
    const u128 inc = ((u128)rng_state[2] << 64) | rng_state[3];
    const uint64_t n8 = (uint64_t)shots * nb;
    const uint64_t base_flip = nb ? ((n8 + 3) / 4 + 1) / 2 : 0;
    std::vector<int32_t> perr(npairs);
    int nerr = 0;
    for (int j = 0; j < npairs; ++j) perr[j] = pair_err[j] >= 0 ? nerr++ : -1;
    if (raw_used) *raw_used = (int64_t)(base_flip + (uint64_t)nerr * shots);
    cudaStream_t st = nullptr;
    LSG_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    auto al = [](size_t v) { return (v + 255) & ~size_t(255); };
    size_t off = 0;
    const size_t o_b = off; off += al(bx.size() * 8);
    const size_t o_x = off; off += al((size_t)W * 8);
    const size_t o_w = off; off += al((size_t)shots * W * 8);
    const size_t o_pp = off; off += al((size_t)npairs * 4);
    const size_t o_pc = off; off += al((size_t)npairs * 4);
    const size_t o_pe = off; off += al((size_t)npairs * 4);
    const size_t o_p0 = off; off += al((size_t)npairs * 8);
    const size_t o_p1 = off; off += al((size_t)npairs * 8);
    const size_t o_out = off; off += al((size_t)shots * nclbits);
    Scratch work;
    int rc = ensure(work, off);
    if (rc != LSG_OK) {
        cudaStreamDestroy(st);
        return rc;
    }
    char* b = (char*)work.ptr;
    cudaError_t ce = cudaSuccess;
    auto H2D = [&](size_t o, const void* src, size_t bytes) {
        if (bytes && ce == cudaSuccess) ce = cudaMemcpyAsync(b + o, src, bytes, cudaMemcpyHostToDevice, st);
    };
    H2D(o_b, bx.data(), bx.size() * 8);
    H2D(o_x, xw.data(), (size_t)W * 8);
    H2D(o_pp, pair_pos, (size_t)npairs * 4);
    H2D(o_pc, pair_clbit, (size_t)npairs * 4);
    H2D(o_pe, perr.data(), (size_t)npairs * 4);
    H2D(o_p0, p01, (size_t)npairs * 8);
    H2D(o_p1, p10, (size_t)npairs * 8);
    if (ce == cudaSuccess) ce = cudaMemsetAsync(b + o_out, 0, (size_t)shots * nclbits, st);
    if (ce == cudaSuccess) {
        k_sampled<<<(unsigned)std::min<int64_t>(shots, 152 * 16), 64, 0, st>>>((const uint64_t*)(b + o_b), nb, W,
                                                                             (const uint64_t*)(b + o_x), (int)shots, s0,
                                                                             inc, (uint64_t*)(b + o_w));
        ce = cudaGetLastError();
    }
    if (ce == cudaSuccess) {
        const int64_t tot = shots * npairs;
        k_words_to_pairs<<<(unsigned)std::max<int64_t>(1, std::min<int64_t>((tot + kS - 1) / kS, 152 * 64)), kS, 0, st>>>(
            (const uint64_t*)(b + o_w), W, (int)shots, npairs, (const int*)(b + o_pp), (const int*)(b + o_pc),
            (const int*)(b + o_pe), (const double*)(b + o_p0), (const double*)(b + o_p1), s0, inc, base_flip, nclbits,
            (uint8_t*)(b + o_out));
        ce = cudaGetLastError();
    }
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(bits_out, b + o_out, (size_t)shots * nclbits, cudaMemcpyDeviceToHost, st);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
    release(work);
    cudaStreamDestroy(st);
    if (ce != cudaSuccess) return fail(LSG_E_CUDA, "stabilizer sampling failed: %s", cudaGetErrorString(ce));
    return LSG_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------------------------
// Dynamic Clifford circuits, one tableau per shot (stabilizer.py:653-694), in Orrery's draw order.
//
// One CTA walks the shots in order. The tableau lives in global memory, qubit-major in 64-bit
// words (word w of qubit q holds rows 64w..64w+63); a shot starts from a copy of the noiseless
// prefix. Thread 0 owns the generator: the PCG64 state, and NumPy's buffered uint32 half, since
// measurements draw integers(2) (the top bit of a uint32) between the doubles of noise and readout.

namespace lsg {

struct ShotOp {
    int16_t code;   // gate code, or 100 measure, 101 reset, 102 if, 103 else, 104 endif
    int16_t noise;  // gate: noise table; measure: readout table (-1: none)
    int16_t a, b, c;
    int16_t clbit;  // measure target (-1: discarded)
    int32_t aux;    // if: condition index; if/else: index to jump to
};

struct ShotCond {
    int32_t n, negate;
    uint64_t value;
    int32_t bits[64];
};

struct RngCtl {
    u128 s, inc;       // current state
    uint64_t pos;      // raw draws so far
    uint32_t has32, buf32;
};

__device__ __forceinline__ uint64_t rng_next64(RngCtl& g) {
    g.s = g.s * pcg_mult() + g.inc;
    g.pos++;
    return pcg_output(g.s);
}

__device__ __forceinline__ double rng_double(RngCtl& g) { return pcg_double(rng_next64(g)); }

__device__ __forceinline__ uint32_t rng_uint32(RngCtl& g) {
    if (g.has32) {
        g.has32 = 0;
        return g.buf32;
    }
    const uint64_t raw = rng_next64(g);
    g.buf32 = (uint32_t)(raw >> 32);
    g.has32 = 1;
    return (uint32_t)raw;
}

// a gate on one 64-row word of a qubit-major tableau (stabilizer.py:224-264)
__device__ __forceinline__ uint64_t tab_gate64(uint64_t* X, uint64_t* Z, int W, int w, const ShotOp& g,
                                               const CTable* tables) {
    const int a = g.a;
    uint64_t& xa = X[(int64_t)a * W + w];
    uint64_t& za = Z[(int64_t)a * W + w];
    uint64_t r = 0;
    switch (g.code) {
        case 0: break;
        case 1: { const uint64_t x = xa; r = x & za; xa = za; za = x; break; }
        case 2: r = xa & za; za ^= xa; break;
        case 3: r = xa & ~za; za ^= xa; break;
        case 4: r = za; break;
        case 5: r = xa ^ za; break;
        case 6: r = xa; break;
        case 7: {
            uint64_t& xb = X[(int64_t)g.b * W + w];
            uint64_t& zb = Z[(int64_t)g.b * W + w];
            r = xa & zb & ~(xb ^ za);
            xb ^= xa;
            za ^= zb;
            break;
        }
        case 8: {
            uint64_t& xb = X[(int64_t)g.b * W + w];
            uint64_t& zb = Z[(int64_t)g.b * W + w];
            r = xa & xb & (za ^ zb);
            za ^= xb;
            zb ^= xa;
            break;
        }
        default: {
            const CTable& t = tables[g.code - 16];
            const int k = t.k;
            const int q[3] = {g.a, g.b, g.c};
            uint64_t nx[3] = {0, 0, 0}, nz[3] = {0, 0, 0};
            for (int j = 0; j < 64; ++j) {
                int idx = 0;
                for (int i = 0; i < k; ++i)
                    idx = (idx << 2) | (int)(((X[(int64_t)q[i] * W + w] >> j) & 1) << 1) | (int)((Z[(int64_t)q[i] * W + w] >> j) & 1);
                const uint8_t e = t.e[idx];
                r |= (uint64_t)(e >> 7) << j;
                for (int i = 0; i < k; ++i) {
                    nx[i] |= (uint64_t)((e >> (2 * (k - 1 - i) + 1)) & 1) << j;
                    nz[i] |= (uint64_t)((e >> (2 * (k - 1 - i))) & 1) << j;
                }
            }
            for (int i = 0; i < k; ++i) {
                X[(int64_t)q[i] * W + w] = nx[i];
                Z[(int64_t)q[i] * W + w] = nz[i];
            }
            break;
        }
    }
    return r;
}

__device__ __forceinline__ int getbit(const uint64_t* M, int W, int q, int row) {
    return (int)((M[(int64_t)q * W + (row >> 6)] >> (row & 63)) & 1);
}

__device__ __forceinline__ void setbit(uint64_t* M, int W, int q, int row, int v) {
    uint64_t& w = M[(int64_t)q * W + (row >> 6)];
    const uint64_t bit = 1ull << (row & 63);
    w = v ? (w | bit) : (w & ~bit);
}

__device__ int block_sum_int(int v) {
    __shared__ int red[32];
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    int out = 0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) out += red[i];
    __syncthreads();
    return out;
}

struct ShotArgs {
    int n, W, nops, ncl_words;
    int64_t shots;
    const ShotOp* ops;
    const ShotCond* conds;
    const CTable* tables;
    const NTable* noise;
    const double* readout;  // pairs (p01, p10)
    const uint64_t *px, *pz, *pr;  // prefix tableau
    uint64_t *X, *Z, *R;           // working tableau
    uint8_t* sx;                   // scratch row for deterministic outcomes: 2n bytes
    uint64_t* out;                 // shots x ncl_words
    RngCtl* rng;                   // in: start state; out: final state
};

// Measure qubit a of the working tableau; thread 0's generator draws when the outcome is random.
__device__ int shot_measure(const ShotArgs& A, int a, RngCtl& g) {
    const int n = A.n, W = A.W;
    uint64_t *X = A.X, *Z = A.Z, *R = A.R;
    __shared__ int pivot;
    __shared__ int outcome;
    if (threadIdx.x == 0) pivot = 0x7fffffff;
    __syncthreads();
    for (int w = threadIdx.x; w < W; w += blockDim.x) {
        uint64_t bits = X[(int64_t)a * W + w];
        // stabilizer rows only: rows >= n
        const int lo = 64 * w;
        if (lo + 63 < n) continue;
        if (lo < n) bits &= ~0ull << (n - lo);
        if (bits) atomicMin(&pivot, lo + __ffsll((long long)bits) - 1);
    }
    __syncthreads();
    const int p = pivot;
    if (p == 0x7fffffff) {
        // deterministic (stabilizer.py:288-301): rowsum the stabilizers of destabilizers with x[a]
        uint8_t* sx = A.sx;
        uint8_t* sz = A.sx + n;
        for (int q = threadIdx.x; q < n; q += blockDim.x) sx[q] = sz[q] = 0;
        __shared__ int sr;
        if (threadIdx.x == 0) sr = 0;
        __syncthreads();
        for (int i = 0; i < n; ++i) {
            if (!getbit(X, W, a, i)) continue;  // uniform across the block
            const int row = i + n;
            int gsum = 0;
            for (int q = threadIdx.x; q < n; q += blockDim.x) {
                const int xs = getbit(X, W, q, row), zs = getbit(Z, W, q, row);
                const int cx = sx[q], cz = sz[q];
                gsum += (xs & zs) * (cz - cx) + (xs & (1 - zs)) * (cz * (2 * cx - 1)) + ((1 - xs) & zs) * (cx * (1 - 2 * cz));
            }
            const int gt = block_sum_int(gsum);
            if (threadIdx.x == 0) {
                const int tot = 2 * sr + 2 * getbit(R, W, 0, row) + gt;
                sr = (((tot % 4) + 4) % 4) == 2 ? 1 : 0;
            }
            for (int q = threadIdx.x; q < n; q += blockDim.x) {
                sx[q] ^= (uint8_t)getbit(X, W, q, row);
                sz[q] ^= (uint8_t)getbit(Z, W, q, row);
            }
            __syncthreads();
        }
        const int out = sr;
        __syncthreads();
        return out;
    }
    // random outcome (stabilizer.py:308-327): rowsum row p into every other row with x[a] set
    const int rp = getbit(R, W, 0, p);
    for (int w = threadIdx.x; w < W; w += blockDim.x) {
        const uint64_t tmask = X[(int64_t)a * W + w] & ~((p >> 6) == w ? (1ull << (p & 63)) : 0ull);
        if (!tmask) continue;
        uint64_t c0 = 0, c1 = 0;  // per-row phase exponent mod 4, bit sliced
        for (int q = 0; q < n; ++q) {
            const int xs = getbit(X, W, q, p), zs = getbit(Z, W, q, p);
            if (!xs && !zs) continue;
            const uint64_t xt = X[(int64_t)q * W + w], zt = Z[(int64_t)q * W + w];
            uint64_t P, M;
            if (xs && zs) {
                P = ~xt & zt;
                M = xt & ~zt;
            } else if (xs) {
                P = xt & zt;
                M = ~xt & zt;
            } else {
                P = xt & ~zt;
                M = xt & zt;
            }
            c1 ^= c0 & P;
            c0 ^= P;
            c1 ^= c0 & M;  // + 3 = + 1 then + 2
            c0 ^= M;
            c1 ^= M;
        }
        const uint64_t rt = R[w];
        const uint64_t rpm = rp ? ~0ull : 0ull;
        const uint64_t newr = ~c0 & (c1 ^ rt ^ rpm);
        R[w] = (rt & ~tmask) | (newr & tmask);
        for (int q = 0; q < n; ++q) {
            if (getbit(X, W, q, p)) X[(int64_t)q * W + w] ^= tmask;
            if (getbit(Z, W, q, p)) Z[(int64_t)q * W + w] ^= tmask;
        }
    }
    __syncthreads();
    // row p-n := row p; row p := Z_a; r[p] := outcome
    for (int q = threadIdx.x; q < n; q += blockDim.x) {
        setbit(X, W, q, p - n, getbit(X, W, q, p));
        setbit(Z, W, q, p - n, getbit(Z, W, q, p));
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        setbit(R, W, 0, p - n, getbit(R, W, 0, p));
        outcome = (int)(rng_uint32(g) >> 31);  // integers(2): top bit of a uint32
    }
    __syncthreads();
    for (int q = threadIdx.x; q < n; q += blockDim.x) {
        setbit(X, W, q, p, 0);
        setbit(Z, W, q, p, q == a ? 1 : 0);
    }
    __syncthreads();
    if (threadIdx.x == 0) setbit(R, W, 0, p, outcome);
    __syncthreads();
    return outcome;
}

__global__ void k_per_shot(ShotArgs A) {
    const int n = A.n, W = A.W;
    __shared__ RngCtl g;
    __shared__ uint64_t clb[4];
    __shared__ int pc_next;
    __shared__ uint32_t racc_all;
    if (threadIdx.x == 0) g = *A.rng;
    __syncthreads();
    const int64_t tw = (int64_t)n * W;
    for (int64_t s = 0; s < A.shots; ++s) {
        for (int64_t i = threadIdx.x; i < tw; i += blockDim.x) {
            A.X[i] = A.px[i];
            A.Z[i] = A.pz[i];
        }
        for (int w = threadIdx.x; w < W; w += blockDim.x) A.R[w] = A.pr[w];
        if (threadIdx.x < 4) clb[threadIdx.x] = 0;
        __syncthreads();
        int pc = 0;
        while (pc < A.nops) {
            const ShotOp op = A.ops[pc];
            int next = pc + 1;
            if (op.code < 100) {
                for (int w = threadIdx.x; w < W; w += blockDim.x) A.R[w] ^= tab_gate64(A.X, A.Z, W, w, op, A.tables);
                __syncthreads();
                if (op.noise >= 0) {
                    const NTable& nt = A.noise[op.noise];
                    __shared__ int pick;
                    if (threadIdx.x == 0) {
                        const double u = rng_double(g);
                        int k = 0;
                        while (k < nt.nb && nt.cum[k] <= u) ++k;
                        pick = k > nt.nb - 1 ? nt.nb - 1 : k;
                    }
                    __syncthreads();
                    const uint8_t lab = nt.label[pick];
                    const int qs[2] = {op.a, op.b};
                    for (int w = threadIdx.x; w < W; w += blockDim.x)
                        for (int qi = 0; qi < nt.k; ++qi) {
                            const int sh = 2 * (nt.k - 1 - qi);
                            if ((lab >> (sh + 1)) & 1) A.R[w] ^= A.Z[(int64_t)qs[qi] * W + w];
                            if ((lab >> sh) & 1) A.R[w] ^= A.X[(int64_t)qs[qi] * W + w];
                        }
                    __syncthreads();
                }
            } else if (op.code == 100 || op.code == 101) {
                int out = shot_measure(A, op.a, g);
                if (op.code == 101) {
                    if (out) {  // X on a after the measurement (Tableau.reset, stabilizer.py:329-331)
                        for (int w = threadIdx.x; w < W; w += blockDim.x) A.R[w] ^= A.Z[(int64_t)op.a * W + w];
                    }
                    __syncthreads();
                } else {
                    if (threadIdx.x == 0) {
                        if (op.noise >= 0) {
                            const double u = rng_double(g);
                            if (u < (out ? A.readout[2 * op.noise + 1] : A.readout[2 * op.noise])) out ^= 1;
                        }
                        if (op.clbit >= 0) {
                            uint64_t& word = clb[op.clbit >> 6];
                            const uint64_t bit = 1ull << (op.clbit & 63);
                            word = out ? (word | bit) : (word & ~bit);
                        }
                    }
                    __syncthreads();
                }
            } else if (op.code == 102) {
                if (threadIdx.x == 0) {
                    const ShotCond& c = A.conds[op.c];
                    uint64_t reading = 0;
                    for (int i = 0; i < c.n; ++i) reading |= ((clb[c.bits[i] >> 6] >> (c.bits[i] & 63)) & 1ull) << i;
                    const bool holds = (reading == c.value) != (c.negate != 0);
                    pc_next = holds ? pc + 1 : op.aux;
                }
                __syncthreads();
                next = pc_next;
                __syncthreads();
            } else if (op.code == 103) {
                next = op.aux;  // the end of the then-branch skips the else-branch
            }
            pc = next;
        }
        if (threadIdx.x < A.ncl_words) A.out[s * A.ncl_words + threadIdx.x] = clb[threadIdx.x];
        __syncthreads();
    }
    (void)racc_all;
    if (threadIdx.x == 0) *A.rng = g;
}

}  // namespace lsg

extern "C" int lsg_per_shot_run(int n, const lsg_cgate* prefix, int64_t nprefix, const lsg_shot_op* ops, int32_t nops,
                                const uint8_t* tables, int32_t ntables, const lsg_noise_table* noise, int32_t nnoise,
                                const double* readout, int32_t nreadout, const lsg_shot_cond* conds, int32_t nconds,
                                int32_t num_clbits, int64_t shots, uint64_t* rng_state, uint64_t* clbits_out) {
    using namespace lsg;
    clear_error();
    if (n < 1 || n > 2048 || nprefix < 0 || nops < 0 || shots < 0 || !rng_state || !clbits_out || num_clbits < 0 ||
        num_clbits > 256 || (nops && !ops) || (nprefix && !prefix))
        return fail(LSG_E_ARG, "lsg_per_shot_run: bad arguments");
    if (shots == 0) return LSG_OK;
    // validate the program
    for (int i = 0; i < nops; ++i) {
        const lsg_shot_op& o = ops[i];
        const bool gate = o.code < 100;
        if (gate) {
            const int k = (o.code == 7 || o.code == 8) ? 2 : (o.code >= 16 ? o.nq : 1);
            if ((o.code > 8 && o.code < 16) || (o.code >= 16 && o.code - 16 >= ntables) || k < 1 || k > 3)
                return fail(LSG_E_ARG, "op %d: bad gate", i);
            const int q[3] = {o.a, o.b, o.c};
            for (int j = 0; j < k; ++j)
                if (q[j] < 0 || q[j] >= n) return fail(LSG_E_ARG, "op %d: bad qubit", i);
            if (o.noise >= nnoise) return fail(LSG_E_ARG, "op %d: bad noise table", i);
        } else if (o.code == 100 || o.code == 101) {
            if (o.a < 0 || o.a >= n || o.clbit >= num_clbits || o.noise >= nreadout) return fail(LSG_E_ARG, "op %d: bad measurement", i);
        } else if (o.code == 102) {
            if (o.c < 0 || o.c >= nconds || o.aux <= i || o.aux > nops) return fail(LSG_E_ARG, "op %d: bad if", i);
        } else if (o.code == 103) {
            if (o.aux <= i || o.aux > nops) return fail(LSG_E_ARG, "op %d: bad else", i);
        } else if (o.code != 104) {
            return fail(LSG_E_ARG, "op %d: unknown code", i);
        }
    }
    for (int i = 0; i < nconds; ++i) {
        if (conds[i].n < 1 || conds[i].n > 64) return fail(LSG_E_ARG, "condition %d is malformed", i);
        for (int j = 0; j < conds[i].n; ++j)
            if (conds[i].bits[j] < 0 || conds[i].bits[j] >= num_clbits) return fail(LSG_E_ARG, "condition %d names a missing bit", i);
    }
    // the prefix tableau, then qubit-major 64-bit words
    lsg_tab t = nullptr;
    LSG_CHECK(lsg_tab_create(n, &t));
    int rc = lsg_tab_apply(t, prefix, nprefix, tables, ntables);
    if (rc != LSG_OK) {
        lsg_tab_free(t);
        return rc;
    }
    const int W = (2 * n + 63) / 64;
    std::vector<uint8_t> hx((size_t)n * 2 * n), hz((size_t)n * 2 * n), hr(2 * n);
    rc = lsg_tab_download(t, hx.data(), hz.data(), hr.data());
    lsg_tab_free(t);
    LSG_CHECK(rc);
    std::vector<uint64_t> px((size_t)n * W, 0), pz((size_t)n * W, 0), pr(W, 0);
    for (int q = 0; q < n; ++q)
        for (int row = 0; row < 2 * n; ++row) {
            if (hx[(size_t)q * 2 * n + row]) px[(size_t)q * W + (row >> 6)] |= 1ull << (row & 63);
            if (hz[(size_t)q * 2 * n + row]) pz[(size_t)q * W + (row >> 6)] |= 1ull << (row & 63);
        }
    for (int row = 0; row < 2 * n; ++row)
        if (hr[row]) pr[row >> 6] |= 1ull << (row & 63);
    std::vector<ShotOp> dops(std::max(nops, 1));
    for (int i = 0; i < nops; ++i)
        dops[i] = ShotOp{ops[i].code, ops[i].noise, ops[i].a, ops[i].b, ops[i].c, ops[i].clbit, ops[i].aux};
    std::vector<ShotCond> dconds(std::max(nconds, 1));
    for (int i = 0; i < nconds; ++i) {
        dconds[i].n = conds[i].n;
        dconds[i].negate = conds[i].negate;
        dconds[i].value = conds[i].value;
        for (int j = 0; j < 64; ++j) dconds[i].bits[j] = conds[i].bits[j];
    }
    std::vector<CTable> ct;
    LSG_CHECK(tables_device(tables, ntables, ct));
    std::vector<NTable> nt(std::max(nnoise, 1));
    for (int i = 0; i < nnoise; ++i) {
        nt[i].k = noise[i].k;
        nt[i].nb = noise[i].nbranch;
        for (int j = 0; j < 16; ++j) {
            nt[i].cum[j] = noise[i].cumulative[j];
            nt[i].label[j] = noise[i].label[j];
        }
    }
    RngCtl g0{};
    g0.s = ((u128)rng_state[0] << 64) | rng_state[1];
    g0.inc = ((u128)rng_state[2] << 64) | rng_state[3];
    g0.pos = 0;
    g0.has32 = (uint32_t)rng_state[4];
    g0.buf32 = (uint32_t)rng_state[5];
    const int words = std::max(1, (num_clbits + 63) / 64);
    auto al = [](size_t v) { return (v + 255) & ~size_t(255); };
    size_t off = 0;
    const size_t tb = (size_t)n * W * 8;
    const size_t o_px = off; off += al(tb);
    const size_t o_pz = off; off += al(tb);
    const size_t o_pr = off; off += al((size_t)W * 8);
    const size_t o_x = off; off += al(tb);
    const size_t o_z = off; off += al(tb);
    const size_t o_r = off; off += al((size_t)W * 8);
    const size_t o_sx = off; off += al((size_t)2 * n);
    const size_t o_ops = off; off += al(dops.size() * sizeof(ShotOp));
    const size_t o_c = off; off += al(dconds.size() * sizeof(ShotCond));
    const size_t o_t = off; off += al(ct.size() * sizeof(CTable));
    const size_t o_n = off; off += al(nt.size() * sizeof(NTable));
    const size_t o_ro = off; off += al((size_t)std::max(nreadout, 1) * 16);
    const size_t o_out = off; off += al((size_t)shots * words * 8);
    const size_t o_g = off; off += al(sizeof(RngCtl));
    Scratch work;
    LSG_CHECK(ensure(work, off));
    char* b = (char*)work.ptr;
    cudaError_t ce = cudaSuccess;
    auto H2D = [&](size_t o, const void* src, size_t bytes) {
        if (bytes && ce == cudaSuccess) ce = cudaMemcpy(b + o, src, bytes, cudaMemcpyHostToDevice);
    };
    H2D(o_px, px.data(), tb);
    H2D(o_pz, pz.data(), tb);
    H2D(o_pr, pr.data(), (size_t)W * 8);
    H2D(o_ops, dops.data(), dops.size() * sizeof(ShotOp));
    H2D(o_c, dconds.data(), dconds.size() * sizeof(ShotCond));
    H2D(o_t, ct.data(), ct.size() * sizeof(CTable));
    H2D(o_n, nt.data(), nt.size() * sizeof(NTable));
    if (nreadout) H2D(o_ro, readout, (size_t)nreadout * 16);
    H2D(o_g, &g0, sizeof(RngCtl));
    ShotArgs A{};
    A.n = n;
    A.W = W;
    A.nops = nops;
    A.ncl_words = words;
    A.shots = shots;
    A.ops = (const ShotOp*)(b + o_ops);
    A.conds = (const ShotCond*)(b + o_c);
    A.tables = (const CTable*)(b + o_t);
    A.noise = (const NTable*)(b + o_n);
    A.readout = (const double*)(b + o_ro);
    A.px = (const uint64_t*)(b + o_px);
    A.pz = (const uint64_t*)(b + o_pz);
    A.pr = (const uint64_t*)(b + o_pr);
    A.X = (uint64_t*)(b + o_x);
    A.Z = (uint64_t*)(b + o_z);
    A.R = (uint64_t*)(b + o_r);
    A.sx = (uint8_t*)(b + o_sx);
    A.out = (uint64_t*)(b + o_out);
    A.rng = (RngCtl*)(b + o_g);
    if (ce == cudaSuccess) {
        k_per_shot<<<1, 512>>>(A);
        ce = cudaGetLastError();
    }
    if (ce == cudaSuccess) ce = cudaDeviceSynchronize();
    std::vector<uint64_t> out((size_t)shots * words);
    RngCtl gend{};
    if (ce == cudaSuccess) ce = cudaMemcpy(out.data(), b + o_out, out.size() * 8, cudaMemcpyDeviceToHost);
    if (ce == cudaSuccess) ce = cudaMemcpy(&gend, b + o_g, sizeof(RngCtl), cudaMemcpyDeviceToHost);
    release(work);
    if (ce != cudaSuccess) return fail(LSG_E_CUDA, "the per-shot run failed: %s", cudaGetErrorString(ce));
    for (int64_t s = 0; s < shots; ++s)
        for (int w = 0; w < 4; ++w) clbits_out[s * 4 + w] = w < words ? out[(size_t)s * words + w] : 0;
    rng_state[0] = (uint64_t)(gend.s >> 64);
    rng_state[1] = (uint64_t)gend.s;
    rng_state[4] = gend.has32;
    rng_state[5] = gend.buf32;
    rng_state[6] = gend.pos;
    return LSG_OK;
}
