// Reductions over a register, all accumulated in FP64 whatever the register's precision, and
// all in a fixed order (block-local trees, then block partials summed in index order) so a
// result never depends on scheduling.
//
//  * probabilities       — Statevector/DensityMatrix.probabilities (engines.py:207-209, :257-260)
//  * sampling            — _sample (simulator.py:254-284): marginal (engines.py:267-275), CDF,
//                          upper-bound search, readout flips
//  * Pauli expectations  — expectation (simulator.py:489-527)
//  * p(1) and collapse   — Statevector.probability_of_one / collapse (engines.py:185-201)
#include <algorithm>
#include <mutex>
#include <vector>

#include "common.cuh"

namespace lsg {

constexpr int kThreads = 256;
constexpr int64_t kMaxGridY = 65535;  // the largest grid y extent of a launch
constexpr int64_t kExpectL2Bytes = 48ll << 20;  // a member group that stays resident in the 126 MiB L2
constexpr int kMaxOutcomePairs = 30;   // outcome space of lsg_outcome_probabilities: 2^30 doubles at most

template <typename R>
__device__ __forceinline__ double norm2(Cx<R> a) {
    return (double)a.re * (double)a.re + (double)a.im * (double)a.im;
}

// fixed-order block sum of one double per thread; result valid in thread 0
__device__ double block_sum(double v) {
    __shared__ double buf[kThreads];
    buf[threadIdx.x] = v;
    __syncthreads();
    for (int s = kThreads / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) buf[threadIdx.x] += buf[threadIdx.x + s];
        __syncthreads();
    }
    double out = buf[0];
    __syncthreads();
    return out;
}

template <typename R>
__global__ void k_probs_sv(const Cx<R>* __restrict__ a, double* __restrict__ out, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = norm2(a[i]);
}

template <typename R>
__global__ void k_probs_dm(const Cx<R>* __restrict__ rho, double* __restrict__ out, int64_t d) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < d; i += (int64_t)gridDim.x * blockDim.x) {
        double v = (double)rho[i * (d + 1)].re;
        out[i] = v > 0.0 ? v : 0.0;
    }
}

__device__ __forceinline__ uint64_t deposit_bits(uint64_t x, const int* pos, int n) {
    uint64_t out = 0;
    for (int j = 0; j < n; ++j) out |= ((x >> j) & 1ull) << pos[j];
    return out;
}

struct BitLists {
    int keep[32];
    int drop[32];
    int nkeep, ndrop;
};

// marginal, few dropped bits: one thread per output, dropped combinations summed in order
__global__ void k_marginal_thread(const double* __restrict__ p, double* __restrict__ dist, BitLists bl) {
    const int64_t nout = 1ll << bl.nkeep;
    const int64_t ninner = 1ll << bl.ndrop;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < nout; j += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t base = deposit_bits((uint64_t)j, bl.keep, bl.nkeep);
        double acc = 0.0;
        for (int64_t r = 0; r < ninner; ++r) acc += p[base | deposit_bits((uint64_t)r, bl.drop, bl.ndrop)];
        dist[j] = acc;
    }
}

// marginal, many dropped bits: one block per output, tree-reduced
__global__ void k_marginal_block(const double* __restrict__ p, double* __restrict__ dist, BitLists bl) {
    const int64_t ninner = 1ll << bl.ndrop;
    for (int64_t j = blockIdx.x; j < (1ll << bl.nkeep); j += gridDim.x) {
        const uint64_t base = deposit_bits((uint64_t)j, bl.keep, bl.nkeep);
        double acc = 0.0;
        for (int64_t r = threadIdx.x; r < ninner; r += blockDim.x) acc += p[base | deposit_bits((uint64_t)r, bl.drop, bl.ndrop)];
        double tot = block_sum(acc);
        if (threadIdx.x == 0) dist[j] = tot;
    }
}

constexpr int kScanPer = 8;  // elements per thread in the scan
constexpr int kScanBlock = kThreads * kScanPer;

__global__ void k_scan_block_sums(const double* __restrict__ x, double* __restrict__ sums, int64_t n) {
    const int64_t start = (int64_t)blockIdx.x * kScanBlock;
    double acc = 0.0;
    for (int i = 0; i < kScanPer; ++i) {
        int64_t k = start + (int64_t)threadIdx.x * kScanPer + i;
        if (k < n) acc += x[k];
    }
    double tot = block_sum(acc);
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

__global__ void k_scan_sums_serial(double* sums, int64_t nblocks) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double run = 0.0;
    for (int64_t b = 0; b < nblocks; ++b) {
        double v = sums[b];
        sums[b] = run;  // exclusive
        run += v;
    }
}

__global__ void k_scan_apply(const double* __restrict__ x, double* __restrict__ out, const double* __restrict__ sums,
                             int64_t n) {
    __shared__ double tsum[kThreads];
    const int64_t start = (int64_t)blockIdx.x * kScanBlock + (int64_t)threadIdx.x * kScanPer;
    double local[kScanPer];
    double acc = 0.0;
    for (int i = 0; i < kScanPer; ++i) {
        int64_t k = start + i;
        acc += (k < n) ? x[k] : 0.0;
        local[i] = acc;
    }
    tsum[threadIdx.x] = acc;
    __syncthreads();
    // inclusive Hillis-Steele over thread totals (fixed order)
    for (int off = 1; off < kThreads; off <<= 1) {
        double v = threadIdx.x >= off ? tsum[threadIdx.x - off] : 0.0;
        __syncthreads();
        tsum[threadIdx.x] += v;
        __syncthreads();
    }
    const double before = sums[blockIdx.x] + (threadIdx.x ? tsum[threadIdx.x - 1] : 0.0);
    for (int i = 0; i < kScanPer; ++i) {
        int64_t k = start + i;
        if (k < n) out[k] = before + local[i];
    }
}

struct PairInfo {
    int pos, has_err, err_index, pad;
    double p01, p10;
};

__global__ void k_search(const double* __restrict__ cum, int64_t n, const double* __restrict__ u, int64_t shots,
                         const PairInfo* __restrict__ pairs, int npairs, const double* __restrict__ flipu,
                         uint8_t* __restrict__ bits, uint8_t* __restrict__ near, unsigned long long* near_count) {
    // the CDF is normalised on the fly: cum[i] / cum[n-1] is the same correctly rounded quotient
    // the reference stores after `cumulative /= cumulative[-1]`
    const double last = cum[n - 1];
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < shots; s += (int64_t)gridDim.x * blockDim.x) {
        const double v = u[s];
        // upper bound: first index with cum[idx] > v
        int64_t lo = 0, hi = n;
        while (lo < hi) {
            int64_t mid = (lo + hi) >> 1;
            if (cum[mid] / last <= v) lo = mid + 1;
            else hi = mid;
        }
        const double tol = 1e-12;
        bool close = (lo < n && fabs(cum[lo] / last - v) < tol) || (lo > 0 && fabs(v - cum[lo - 1] / last) < tol);
        if (near) near[s] = close ? 1 : 0;
        if (close) atomicAdd(near_count, 1ull);
        const int64_t idx = lo < n ? lo : n - 1;
        for (int j = 0; j < npairs; ++j) {
            const PairInfo pi = pairs[j];
            int bit = (int)((idx >> pi.pos) & 1);
            if (pi.has_err) {
                const double r = flipu[(int64_t)pi.err_index * shots + s];
                if (r < (bit ? pi.p10 : pi.p01)) bit ^= 1;
            }
            bits[s * npairs + j] = (uint8_t)bit;
        }
    }
}

// Exact outcomes with readout error. Pair j of the final measurements reads measured position
// pos[j]; the outcome space has one bit per pair (bit j = what pair j reported).
struct PairPositions {
    int pos[64];
    int n;
};

// E[e(i)] = dist[i] (0 where dist[i] <= threshold: those indices are left out, as the reference
// skips them), e(i) = the pair bits index i gives before any flip. E is zero elsewhere (the pair
// bits of two pairs on one qubit agree).
__global__ void k_pair_scatter(const double* __restrict__ dist, int64_t nd, PairPositions pp, double threshold,
                               double* __restrict__ e_out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nd; i += (int64_t)gridDim.x * blockDim.x) {
        uint64_t e = 0;
        for (int j = 0; j < pp.n; ++j) e |= (uint64_t)((i >> pp.pos[j]) & 1) << j;
        const double v = dist[i];
        e_out[e] = v > threshold ? v : 0.0;
    }
}

// Pair j's readout error on the outcome space: a reported 0 becomes 1 with p01, a 1 becomes 0
// with p10 (a column-stochastic 2x2 on bit j).
__global__ void k_readout_flip(double* __restrict__ e, int64_t ne, int j, double p01, double p10) {
    const uint64_t bit = 1ull << j;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < (ne >> 1); t += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t lo = (uint64_t)t & (bit - 1);
        const uint64_t i0 = (((uint64_t)t >> j) << (j + 1)) | lo, i1 = i0 | bit;
        const double a0 = e[i0], a1 = e[i1];
        e[i0] = a0 * (1.0 - p01) + a1 * p10;
        e[i1] = a0 * p01 + a1 * (1.0 - p10);
    }
}

// Re(i^ny * conj(a[i ^ x]) * a[i]) * (-1)^|i & z|: one Pauli string's summand at index i, in R
template <typename R>
__device__ __forceinline__ R pauli_summand(const Cx<R>* __restrict__ s, uint64_t i, uint64_t x, uint64_t z, int ny) {
    const Cx<R> va = s[i], vb = s[i ^ x];
    const R wr = vb.re * va.re + vb.im * va.im;  // conj(b) * a
    const R wi = vb.re * va.im - vb.im * va.re;
    R term = ny == 0 ? wr : ny == 1 ? -wi : ny == 2 ? -wr : wi;
    return (__popcll(i & z) & 1) ? -term : term;
}

// <P> partial sums for every member (grid.y) and term: partials[(member * nterms + t) * gridDim.x + block].
// Statevectors: P is Hermitian, so the summands at i and i ^ x are equal; each pair is read once,
// from the half of the indices with x's top bit clear, and counted twice (x = 0 sums every
// index once). Summands are formed in the register's precision and added four at a time before
// the FP64 accumulation. Density matrices (dm_n > 0): the summands are the diagonal-block
// entries rho[i, i ^ x], in FP64.
template <typename R>
__global__ void k_expect(const Cx<R>* __restrict__ a, int64_t elems, int dm_n, const uint64_t* __restrict__ xm,
                         const uint64_t* __restrict__ zm, int nterms, double* __restrict__ partials) {
    const int64_t member = blockIdx.y;
    const Cx<R>* s = a + member * elems;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t first = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    for (int t = 0; t < nterms; ++t) {
        const uint64_t x = xm[t], z = zm[t];
        const int ny = __popcll(x & z) & 3;
        double acc = 0.0;
        if (dm_n) {
            const int64_t count = 1ll << dm_n;
            for (int64_t i = first; i < count; i += stride) {
                const Cx<R> r = s[((uint64_t)i << dm_n) | ((uint64_t)i ^ x)];
                const double wr = r.re, wi = r.im;
                double term = ny == 0 ? wr : ny == 1 ? -wi : ny == 2 ? -wr : wi;
                if (__popcll((uint64_t)i & z) & 1) term = -term;
                acc += term;
            }
        } else {
            const int h = x ? 63 - __clzll((long long)x) : 64;  // x's top bit (none for x = 0)
            const uint64_t low = h < 64 ? (1ull << h) - 1 : ~0ull;
            const int64_t count = x ? elems >> 1 : elems;
            auto index = [&](int64_t j) -> uint64_t {  // the j-th index with bit h clear
                return h < 64 ? ((((uint64_t)j & ~low) << 1) | ((uint64_t)j & low)) : (uint64_t)j;
            };
            int64_t j = first;
            for (; j + 3 * stride < count; j += 4 * stride) {
                R part = pauli_summand(s, index(j), x, z, ny);
                part += pauli_summand(s, index(j + stride), x, z, ny);
                part += pauli_summand(s, index(j + 2 * stride), x, z, ny);
                part += pauli_summand(s, index(j + 3 * stride), x, z, ny);
                acc += (double)part;
            }
            for (; j < count; j += stride) acc += (double)pauli_summand(s, index(j), x, z, ny);
            if (x) acc *= 2.0;
        }
        double tot = block_sum(acc);
        if (threadIdx.x == 0) partials[(member * nterms + t) * gridDim.x + blockIdx.x] = tot;
    }
}

// one block per row: out[row] = sum of partials[row * ncols .. + ncols) in a fixed order
__global__ void k_sum_rows(const double* __restrict__ partials, int64_t ncols, int64_t nrows, double* __restrict__ out) {
    for (int64_t row = blockIdx.x; row < nrows; row += gridDim.x) {
        double acc = 0.0;
        for (int64_t c = threadIdx.x; c < ncols; c += blockDim.x) acc += partials[row * ncols + c];
        double tot = block_sum(acc);
        if (threadIdx.x == 0) out[row] = tot;
    }
}

template <typename R>
__global__ void k_prob_one(const Cx<R>* __restrict__ a, int64_t elems, int q, double* __restrict__ partials) {
    const int64_t half = elems >> 1;
    double acc = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < half; i += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t lo = (uint64_t)i & ((1ull << q) - 1);
        const uint64_t idx = (((uint64_t)i >> q) << (q + 1)) | (1ull << q) | lo;
        acc += norm2(a[idx]);
    }
    double tot = block_sum(acc);
    if (threadIdx.x == 0) partials[blockIdx.x] = tot;
}

template <typename R>
__global__ void k_collapse(Cx<R>* __restrict__ a, int64_t elems, int q, int outcome, double scale_div, int do_scale) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < elems; i += (int64_t)gridDim.x * blockDim.x) {
        const int bit = (int)(((uint64_t)i >> q) & 1);
        if (bit != outcome) {
            a[i] = Cx<R>(R(0), R(0));
        } else if (do_scale) {
            Cx<R> v = a[i];
            a[i] = Cx<R>((R)((double)v.re / scale_div), (R)((double)v.im / scale_div));
        }
    }
}

// Probabilities of Pauli-transfer members: p(s) = 2^-n sum_z r[z] (-1)^{|z & s|} over the 2^n
// diagonal coefficients (register indices below 2^n), a Walsh-Hadamard transform done in FP64 in
// shared memory, one CTA per member, in a fixed butterfly order. Clipped at 0 like the diagonal.
template <typename R>
__global__ void k_probs_ptm(const R* __restrict__ r, int64_t elems, int n, int64_t member0, double* __restrict__ out) {
    extern __shared__ double w[];
    const int64_t member = member0 + blockIdx.x;
    const R* src = r + member * elems;
    const int d = 1 << n;
    for (int i = threadIdx.x; i < d; i += blockDim.x) w[i] = (double)src[i];
    __syncthreads();
    for (int h = 1; h < d; h <<= 1) {
        for (int j = threadIdx.x; j < d / 2; j += blockDim.x) {
            const int i0 = ((j / h) * 2 * h) + (j % h), i1 = i0 + h;
            const double a = w[i0], b = w[i1];
            w[i0] = a + b;
            w[i1] = a - b;
        }
        __syncthreads();
    }
    const double scale = 1.0 / (double)d;
    double* dst = out + (int64_t)blockIdx.x * d;
    for (int i = threadIdx.x; i < d; i += blockDim.x) {
        const double v = w[i] * scale;
        dst[i] = v > 0.0 ? v : 0.0;
    }
}

// <P> of Pauli-transfer members: the coefficient itself, at register index (x << n) | z.
template <typename R>
__global__ void k_expect_ptm(const R* __restrict__ r, int64_t elems, int n, const uint64_t* __restrict__ xm,
                             const uint64_t* __restrict__ zm, int nterms, int64_t batch, double* __restrict__ out) {
    const int64_t total = (int64_t)nterms * batch;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t b = i / nterms;
        const int t = (int)(i - b * nterms);
        out[i] = (double)r[b * elems + (int64_t)((xm[t] << n) | zm[t])];
    }
}

static int launch_probs_ptm(lsg_state_s* s, int n, int64_t member0, int64_t members, double* dev_out) {
    const size_t smem = (size_t)8 << n;
    static std::mutex mu;
    static bool done[3][64] = {};
    int dev = 0;
    LSG_CUDA(cudaGetDevice(&dev));
    const int which = s->precision == LSG_R64 ? 0 : s->precision == LSG_RD ? 2 : 1;
    if (smem > 48 * 1024) {
        std::lock_guard<std::mutex> lock(mu);
        if (dev >= 0 && dev < 64 && !done[which][dev]) {
            if (which == 0)
                LSG_CUDA(cudaFuncSetAttribute(k_probs_ptm<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, 8 << 14));
            else if (which == 2)
                LSG_CUDA(cudaFuncSetAttribute(k_probs_ptm<DF>, cudaFuncAttributeMaxDynamicSharedMemorySize, 8 << 14));
            else
                LSG_CUDA(cudaFuncSetAttribute(k_probs_ptm<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, 8 << 14));
            done[which][dev] = true;
        }
    }
    if (which == 0)
        k_probs_ptm<double><<<(unsigned)members, 512, smem, s->stream>>>((const double*)s->data, s->elems, n, member0, dev_out);
    else if (which == 2)
        k_probs_ptm<DF><<<(unsigned)members, 512, smem, s->stream>>>((const DF*)s->data, s->elems, n, member0, dev_out);
    else
        k_probs_ptm<float><<<(unsigned)members, 512, smem, s->stream>>>((const float*)s->data, s->elems, n, member0, dev_out);
    LSG_CUDA(cudaGetLastError());
    return LSG_OK;
}

static unsigned reduce_grid(int64_t n) {
    int64_t g = (n + kThreads - 1) / kThreads;
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>(g, 152 * 8));
}

// Probabilities of one member into a device buffer of 2^n doubles.
static int probs_device(lsg_state_s* s, int dm_n, int64_t member, double* dev_out, int64_t* n_out) {
    if (member < 0 || member >= s->batch) return fail(LSG_E_ARG, "member %lld out of range", (long long)member);
    if (s->real()) {
        if (2 * dm_n != s->nbits) return fail(LSG_E_STATE, "a Pauli-transfer register of %d bits holds %d qubits", s->nbits, s->nbits / 2);
        if (dm_n > 14) return fail(LSG_E_CAPACITY, "Pauli-transfer probabilities up to 14 qubits");
        LSG_CHECK(launch_probs_ptm(s, dm_n, member, 1, dev_out));
        *n_out = 1ll << dm_n;
        return LSG_OK;
    }
    if (dm_n) {
        if (2 * dm_n != s->nbits) return fail(LSG_E_STATE, "a %d-qubit density register needs %d bits", dm_n, 2 * dm_n);
        const int64_t d = 1ll << dm_n;
        if (s->precision == LSG_C128)
            k_probs_dm<double><<<reduce_grid(d), kThreads, 0, s->stream>>>((const Cx<double>*)s->data + member * s->elems, dev_out, d);
        else
            k_probs_dm<float><<<reduce_grid(d), kThreads, 0, s->stream>>>((const Cx<float>*)s->data + member * s->elems, dev_out, d);
        *n_out = d;
    } else {
        const int64_t n = s->elems;
        if (s->precision == LSG_C128)
            k_probs_sv<double><<<reduce_grid(n), kThreads, 0, s->stream>>>((const Cx<double>*)s->data + member * n, dev_out, n);
        else
            k_probs_sv<float><<<reduce_grid(n), kThreads, 0, s->stream>>>((const Cx<float>*)s->data + member * n, dev_out, n);
        *n_out = n;
    }
    LSG_CUDA(cudaGetLastError());
    return LSG_OK;
}

}  // namespace lsg

using namespace lsg;

extern "C" {

int lsg_probabilities(lsg_state s, int dm_qubits, int64_t member, double* out) {
    clear_error();
    if (!s || !out) return fail(LSG_E_ARG, "null argument");
    if (s->real() && 2 * dm_qubits != s->nbits)
        return fail(LSG_E_STATE, "a Pauli-transfer register of %d bits holds %d qubits", s->nbits, s->nbits / 2);
    const int64_t n = dm_qubits ? (1ll << dm_qubits) : s->elems;
    if (member < 0) {  // every member, one after another in `out`
        LSG_CHECK(ensure(s->scratch, (size_t)n * 8 * s->batch));
        if (s->real() && 2 * dm_qubits == s->nbits && dm_qubits <= 14) {  // one launch for all members
            LSG_CHECK(launch_probs_ptm(s, dm_qubits, 0, s->batch, (double*)s->scratch.ptr));
        } else {
            for (int64_t b = 0; b < s->batch; ++b) {
                int64_t got = 0;
                LSG_CHECK(probs_device(s, dm_qubits, b, (double*)s->scratch.ptr + b * n, &got));
            }
        }
        LSG_CUDA(cudaMemcpyAsync(out, s->scratch.ptr, (size_t)n * 8 * s->batch, cudaMemcpyDeviceToHost, s->stream));
        LSG_CUDA(cudaStreamSynchronize(s->stream));
        return LSG_OK;
    }
    LSG_CHECK(ensure(s->scratch, (size_t)n * 8));
    int64_t got = 0;
    LSG_CHECK(probs_device(s, dm_qubits, member, (double*)s->scratch.ptr, &got));
    LSG_CUDA(cudaMemcpyAsync(out, s->scratch.ptr, (size_t)got * 8, cudaMemcpyDeviceToHost, s->stream));
    LSG_CUDA(cudaStreamSynchronize(s->stream));
    return LSG_OK;
}

int lsg_sample(lsg_state s, int dm_qubits, int64_t member, const int32_t* measured, int32_t m, const double* uniforms,
               int64_t shots, int32_t npairs, const int32_t* pair_pos, const int32_t* pair_has_err,
               const double* pair_p01, const double* pair_p10, const double* flip_uniforms, uint8_t* bits_out,
               uint8_t* near_out, int64_t* near_count) {
    clear_error();
    if (!s || !measured || !uniforms || !bits_out || shots < 0 || npairs < 0 || m < 1)
        return fail(LSG_E_ARG, "lsg_sample: bad arguments");
    if (npairs > 0 && (!pair_pos || !pair_has_err || !pair_p01 || !pair_p10))
        return fail(LSG_E_ARG, "lsg_sample: pair arrays missing");
    const int nq = dm_qubits ? dm_qubits : s->nbits;
    if (m > nq) return fail(LSG_E_ARG, "lsg_sample: more measured qubits than the register has");
    BitLists bl{};
    uint64_t keepmask = 0;
    for (int i = 0; i < m; ++i) {
        if (measured[i] < 0 || measured[i] >= nq || (i && measured[i] <= measured[i - 1]))
            return fail(LSG_E_ARG, "lsg_sample: measured qubits must be ascending and in range");
        bl.keep[i] = measured[i];
        keepmask |= 1ull << measured[i];
    }
    bl.nkeep = m;
    for (int q = 0; q < nq; ++q)
        if (!((keepmask >> q) & 1)) bl.drop[bl.ndrop++] = q;
    int nerr = 0;
    std::vector<PairInfo> pinfo(npairs);
    for (int j = 0; j < npairs; ++j) {
        if (pair_pos[j] < 0 || pair_pos[j] >= m) return fail(LSG_E_ARG, "lsg_sample: pair position out of range");
        pinfo[j] = PairInfo{pair_pos[j], pair_has_err[j] ? 1 : 0, pair_has_err[j] ? nerr : 0, 0, pair_p01[j], pair_p10[j]};
        if (pair_has_err[j]) ++nerr;
    }
    if (nerr && !flip_uniforms) return fail(LSG_E_ARG, "lsg_sample: flip uniforms missing");
    const int64_t nfull = 1ll << nq;
    const int64_t nd = 1ll << m;
    const int64_t nblk = (nd + kScanBlock - 1) / kScanBlock;
    // scratch layout: probs | dist | cum | block sums | uniforms | flip uniforms | pairs | bits | near | count
    size_t off = 0;
    auto take = [&](size_t bytes) {
        size_t at = off;
        off += (bytes + 255) & ~size_t(255);
        return at;
    };
    const size_t o_p = take(nfull * 8), o_d = take(nd * 8), o_c = take(nd * 8), o_b = take(nblk * 8);
    const size_t o_u = take(shots * 8), o_f = take((size_t)nerr * shots * 8), o_pi = take(npairs * sizeof(PairInfo));
    const size_t o_bits = take((size_t)shots * npairs), o_near = take(shots), o_cnt = take(8);
    LSG_CHECK(ensure(s->scratch, off));
    char* base = (char*)s->scratch.ptr;
    double* p = (double*)(base + o_p);
    double* dist = (double*)(base + o_d);
    double* cum = (double*)(base + o_c);
    double* bsum = (double*)(base + o_b);
    int64_t got = 0;
    LSG_CHECK(probs_device(s, dm_qubits, member, p, &got));
    if (m == nq) {
        dist = p;  // every qubit measured, ascending: the marginal is the distribution itself
    } else if (bl.ndrop <= 6) {
        k_marginal_thread<<<reduce_grid(nd), kThreads, 0, s->stream>>>(p, dist, bl);
    } else {
        k_marginal_block<<<(unsigned)std::min<int64_t>(nd, 152 * 16), kThreads, 0, s->stream>>>(p, dist, bl);
    }
    k_scan_block_sums<<<(unsigned)nblk, kThreads, 0, s->stream>>>(dist, bsum, nd);
    k_scan_sums_serial<<<1, 32, 0, s->stream>>>(bsum, nblk);
    k_scan_apply<<<(unsigned)nblk, kThreads, 0, s->stream>>>(dist, cum, bsum, nd);
    LSG_CUDA(cudaGetLastError());
    if (shots > 0) {
        LSG_CUDA(cudaMemcpyAsync(base + o_u, uniforms, shots * 8, cudaMemcpyHostToDevice, s->stream));
        if (nerr)
            LSG_CUDA(cudaMemcpyAsync(base + o_f, flip_uniforms, (size_t)nerr * shots * 8, cudaMemcpyHostToDevice, s->stream));
        if (npairs)
            LSG_CUDA(cudaMemcpyAsync(base + o_pi, pinfo.data(), npairs * sizeof(PairInfo), cudaMemcpyHostToDevice, s->stream));
        LSG_CUDA(cudaMemsetAsync(base + o_cnt, 0, 8, s->stream));
        k_search<<<reduce_grid(shots), kThreads, 0, s->stream>>>(cum, nd, (const double*)(base + o_u), shots,
                                                                 (const PairInfo*)(base + o_pi), npairs,
                                                                 (const double*)(base + o_f), (uint8_t*)(base + o_bits),
                                                                 (uint8_t*)(base + o_near),
                                                                 (unsigned long long*)(base + o_cnt));
        LSG_CUDA(cudaGetLastError());
        if (npairs)
            LSG_CUDA(cudaMemcpyAsync(bits_out, base + o_bits, (size_t)shots * npairs, cudaMemcpyDeviceToHost, s->stream));
        if (near_out) LSG_CUDA(cudaMemcpyAsync(near_out, base + o_near, shots, cudaMemcpyDeviceToHost, s->stream));
        unsigned long long cnt = 0;
        LSG_CUDA(cudaMemcpyAsync(&cnt, base + o_cnt, 8, cudaMemcpyDeviceToHost, s->stream));
        LSG_CUDA(cudaStreamSynchronize(s->stream));
        if (near_count) *near_count = (int64_t)cnt;
    } else {
        LSG_CUDA(cudaStreamSynchronize(s->stream));
        if (near_count) *near_count = 0;
    }
    return LSG_OK;
}

int lsg_outcome_probabilities(lsg_state s, int dm_qubits, const int32_t* measured, int32_t m, int32_t npairs,
                              const int32_t* pair_pos, const double* pair_p01, const double* pair_p10, double threshold,
                              double* out) {
    clear_error();
    if (!s || !measured || !out || m < 1 || npairs < 1 || !pair_pos || !pair_p01 || !pair_p10)
        return fail(LSG_E_ARG, "lsg_outcome_probabilities: bad arguments");
    if (npairs > kMaxOutcomePairs)
        return fail(LSG_E_CAPACITY, "lsg_outcome_probabilities: %d measurement pairs; at most %d", npairs, kMaxOutcomePairs);
    const int nq = dm_qubits ? dm_qubits : s->nbits;
    if (m > nq || m > npairs) return fail(LSG_E_ARG, "lsg_outcome_probabilities: more measured qubits than pairs or qubits");
    BitLists bl{};
    uint64_t keepmask = 0;
    for (int i = 0; i < m; ++i) {
        if (measured[i] < 0 || measured[i] >= nq || (i && measured[i] <= measured[i - 1]))
            return fail(LSG_E_ARG, "lsg_outcome_probabilities: measured qubits must be ascending and in range");
        bl.keep[i] = measured[i];
        keepmask |= 1ull << measured[i];
    }
    bl.nkeep = m;
    for (int q = 0; q < nq; ++q)
        if (!((keepmask >> q) & 1)) bl.drop[bl.ndrop++] = q;
    PairPositions pp{};
    pp.n = npairs;
    uint64_t seen = 0;
    for (int j = 0; j < npairs; ++j) {
        if (pair_pos[j] < 0 || pair_pos[j] >= m) return fail(LSG_E_ARG, "lsg_outcome_probabilities: pair position out of range");
        if (!(pair_p01[j] >= 0 && pair_p01[j] <= 1 && pair_p10[j] >= 0 && pair_p10[j] <= 1))
            return fail(LSG_E_ARG, "lsg_outcome_probabilities: flip probabilities must lie in [0, 1]");
        pp.pos[j] = pair_pos[j];
        seen |= 1ull << pair_pos[j];
    }
    if (seen != (m >= 64 ? ~0ull : (1ull << m) - 1))
        return fail(LSG_E_ARG, "lsg_outcome_probabilities: every measured qubit needs a pair");
    const int64_t nfull = 1ll << nq, nd = 1ll << m, ne = 1ll << npairs;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        size_t at = off;
        off += (bytes + 255) & ~size_t(255);
        return at;
    };
    const size_t o_p = take(nfull * 8), o_d = take(nd * 8), o_e = take(ne * 8);
    LSG_CHECK(ensure(s->scratch, off));
    char* base = (char*)s->scratch.ptr;
    double* p = (double*)(base + o_p);
    double* dist = (double*)(base + o_d);
    double* e = (double*)(base + o_e);
    int64_t got = 0;
    LSG_CHECK(probs_device(s, dm_qubits, 0, p, &got));
    if (m == nq) dist = p;
    else if (bl.ndrop <= 6) k_marginal_thread<<<reduce_grid(nd), kThreads, 0, s->stream>>>(p, dist, bl);
    else k_marginal_block<<<(unsigned)std::min<int64_t>(nd, 152 * 16), kThreads, 0, s->stream>>>(p, dist, bl);
    LSG_CUDA(cudaMemsetAsync(e, 0, (size_t)ne * 8, s->stream));
    k_pair_scatter<<<reduce_grid(nd), kThreads, 0, s->stream>>>(dist, nd, pp, threshold, e);
    for (int j = 0; j < npairs; ++j)
        if (pair_p01[j] != 0.0 || pair_p10[j] != 0.0)
            k_readout_flip<<<reduce_grid(ne >> 1), kThreads, 0, s->stream>>>(e, ne, j, pair_p01[j], pair_p10[j]);
    LSG_CUDA(cudaGetLastError());
    LSG_CUDA(cudaMemcpyAsync(out, e, (size_t)ne * 8, cudaMemcpyDeviceToHost, s->stream));
    LSG_CUDA(cudaStreamSynchronize(s->stream));
    return LSG_OK;
}

int lsg_expect_pauli(lsg_state s, int dm_qubits, const uint64_t* xmask, const uint64_t* zmask, int32_t nterms,
                     double* out) {
    clear_error();
    if (!s || nterms < 0 || (nterms && (!xmask || !zmask || !out))) return fail(LSG_E_ARG, "lsg_expect_pauli: bad arguments");
    if (dm_qubits && 2 * dm_qubits != s->nbits) return fail(LSG_E_STATE, "density register size mismatch");
    if (nterms == 0) return LSG_OK;
    const int nq = dm_qubits ? dm_qubits : s->nbits;
    const uint64_t limit = nq >= 64 ? ~0ull : ((1ull << nq) - 1);
    for (int t = 0; t < nterms; ++t)
        if ((xmask[t] | zmask[t]) & ~limit) return fail(LSG_E_ARG, "lsg_expect_pauli: term %d names a missing qubit", t);
    if (s->real()) {  // Pauli-transfer register: each expectation is one coefficient
        if (2 * dm_qubits != s->nbits) return fail(LSG_E_STATE, "a Pauli-transfer register of %d bits holds %d qubits", s->nbits, s->nbits / 2);
        const int64_t rows = (int64_t)nterms * s->batch;
        const size_t o_x = 0, o_z = ((size_t)nterms * 8 + 255) & ~size_t(255), o_out = 2 * o_z;
        LSG_CHECK(ensure(s->scratch, o_out + (size_t)rows * 8));
        char* base = (char*)s->scratch.ptr;
        LSG_CUDA(cudaMemcpyAsync(base + o_x, xmask, nterms * 8, cudaMemcpyHostToDevice, s->stream));
        LSG_CUDA(cudaMemcpyAsync(base + o_z, zmask, nterms * 8, cudaMemcpyHostToDevice, s->stream));
        if (s->precision == LSG_R64)
            k_expect_ptm<double><<<reduce_grid(rows), kThreads, 0, s->stream>>>(
                (const double*)s->data, s->elems, dm_qubits, (const uint64_t*)(base + o_x), (const uint64_t*)(base + o_z),
                nterms, s->batch, (double*)(base + o_out));
        else if (s->precision == LSG_RD)
            k_expect_ptm<DF><<<reduce_grid(rows), kThreads, 0, s->stream>>>(
                (const DF*)s->data, s->elems, dm_qubits, (const uint64_t*)(base + o_x), (const uint64_t*)(base + o_z),
                nterms, s->batch, (double*)(base + o_out));
        else
            k_expect_ptm<float><<<reduce_grid(rows), kThreads, 0, s->stream>>>(
                (const float*)s->data, s->elems, dm_qubits, (const uint64_t*)(base + o_x), (const uint64_t*)(base + o_z),
                nterms, s->batch, (double*)(base + o_out));
        LSG_CUDA(cudaGetLastError());
        std::vector<double> tmp((size_t)rows);
        LSG_CUDA(cudaMemcpyAsync(tmp.data(), base + o_out, tmp.size() * 8, cudaMemcpyDeviceToHost, s->stream));
        LSG_CUDA(cudaStreamSynchronize(s->stream));
        for (int64_t b = 0; b < s->batch; ++b)
            for (int t = 0; t < nterms; ++t) out[(int64_t)t * s->batch + b] = tmp[b * nterms + t];
        return LSG_OK;
    }
    const int64_t count = dm_qubits ? (1ll << dm_qubits) : s->elems;
    // Statevector members go through in groups small enough to stay in L2 while every term reads
    // them (one group per launch); density-matrix diagonals are small and go all at once.
    const int64_t member_bytes = s->elems * (s->precision == LSG_C128 ? 16 : 8);
    const int64_t chunk = dm_qubits ? kMaxGridY
                                    : std::min<int64_t>(kMaxGridY, std::max<int64_t>(1, kExpectL2Bytes / member_bytes));
    const unsigned grid = std::max(1u, std::min(reduce_grid(count),
                                                (unsigned)std::max<int64_t>(1, 4096 / std::min(chunk, s->batch))));
    size_t off = 0;
    auto take = [&](size_t bytes) {
        size_t at = off;
        off += (bytes + 255) & ~size_t(255);
        return at;
    };
    const int64_t rows = (int64_t)nterms * s->batch;
    const size_t o_x = take(nterms * 8), o_z = take(nterms * 8), o_part = take((size_t)rows * grid * 8),
                 o_out = take((size_t)rows * 8);
    LSG_CHECK(ensure(s->scratch, off));
    char* base = (char*)s->scratch.ptr;
    LSG_CUDA(cudaMemcpyAsync(base + o_x, xmask, nterms * 8, cudaMemcpyHostToDevice, s->stream));
    LSG_CUDA(cudaMemcpyAsync(base + o_z, zmask, nterms * 8, cudaMemcpyHostToDevice, s->stream));
    // members go on grid y, at most 65,535 (or one L2-sized group) per launch
    for (int64_t b0 = 0; b0 < s->batch; b0 += chunk) {
        const int64_t nb = std::min<int64_t>(chunk, s->batch - b0);
        const dim3 g2(grid, (unsigned)nb);
        double* part = (double*)(base + o_part) + b0 * nterms * (int64_t)grid;
        if (s->precision == LSG_C128)
            k_expect<double><<<g2, kThreads, 0, s->stream>>>((const Cx<double>*)s->data + b0 * s->elems, s->elems,
                                                            dm_qubits, (const uint64_t*)(base + o_x),
                                                            (const uint64_t*)(base + o_z), nterms, part);
        else
            k_expect<float><<<g2, kThreads, 0, s->stream>>>((const Cx<float>*)s->data + b0 * s->elems, s->elems,
                                                           dm_qubits, (const uint64_t*)(base + o_x),
                                                           (const uint64_t*)(base + o_z), nterms, part);
    }
    k_sum_rows<<<(unsigned)std::min<int64_t>(rows, 152 * 16), kThreads, 0, s->stream>>>((const double*)(base + o_part), grid,
                                                                                      rows, (double*)(base + o_out));
    LSG_CUDA(cudaGetLastError());
    std::vector<double> tmp((size_t)rows);
    LSG_CUDA(cudaMemcpyAsync(tmp.data(), base + o_out, tmp.size() * 8, cudaMemcpyDeviceToHost, s->stream));
    LSG_CUDA(cudaStreamSynchronize(s->stream));
    for (int64_t b = 0; b < s->batch; ++b)
        for (int t = 0; t < nterms; ++t) out[(int64_t)t * s->batch + b] = tmp[b * nterms + t];
    return LSG_OK;
}

int lsg_prob_one(lsg_state s, int qubit, int64_t member, double* out) {
    clear_error();
    if (!s || !out) return fail(LSG_E_ARG, "null argument");
    if (s->real()) return fail(LSG_E_STATE, "lsg_prob_one takes a statevector register");
    if (qubit < 0 || qubit >= s->nbits) return fail(LSG_E_ARG, "qubit %d out of range", qubit);
    if (member < 0 || member >= s->batch) return fail(LSG_E_ARG, "member out of range");
    const unsigned grid = reduce_grid(s->elems >> 1);
    LSG_CHECK(ensure(s->scratch, (size_t)(grid + 1) * 8));
    double* part = (double*)s->scratch.ptr;
    if (s->precision == LSG_C128)
        k_prob_one<double><<<grid, kThreads, 0, s->stream>>>((const Cx<double>*)s->data + member * s->elems, s->elems, qubit, part);
    else
        k_prob_one<float><<<grid, kThreads, 0, s->stream>>>((const Cx<float>*)s->data + member * s->elems, s->elems, qubit, part);
    k_sum_rows<<<1, kThreads, 0, s->stream>>>(part, grid, (int64_t)1, part + grid);
    LSG_CUDA(cudaGetLastError());
    LSG_CUDA(cudaMemcpyAsync(out, part + grid, 8, cudaMemcpyDeviceToHost, s->stream));
    LSG_CUDA(cudaStreamSynchronize(s->stream));
    return LSG_OK;
}

int lsg_collapse(lsg_state s, int qubit, int outcome, double probability, int64_t member) {
    clear_error();
    if (s && s->real()) return fail(LSG_E_STATE, "lsg_collapse takes a statevector register");
    if (!s) return fail(LSG_E_ARG, "null register");
    if (qubit < 0 || qubit >= s->nbits || (outcome != 0 && outcome != 1)) return fail(LSG_E_ARG, "bad qubit or outcome");
    if (member < 0 || member >= s->batch) return fail(LSG_E_ARG, "member out of range");
    const double div = probability > 0 ? sqrt(probability) : 1.0;
    const int do_scale = probability > 0 ? 1 : 0;
    if (s->precision == LSG_C128)
        k_collapse<double><<<reduce_grid(s->elems), kThreads, 0, s->stream>>>((Cx<double>*)s->data + member * s->elems,
                                                                              s->elems, qubit, outcome, div, do_scale);
    else
        k_collapse<float><<<reduce_grid(s->elems), kThreads, 0, s->stream>>>((Cx<float>*)s->data + member * s->elems,
                                                                             s->elems, qubit, outcome, div, do_scale);
    LSG_CUDA(cudaGetLastError());
    LSG_CUDA(cudaStreamSynchronize(s->stream));
    return LSG_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------------------------
// Allocation-free Pauli expectations.
//
// For callers that cannot let a library allocate device memory: a serving runtime or a host
// framework that owns every byte of the GPU through its own pool (and must keep a hard memory
// budget), or a latency-sensitive loop that cannot afford cudaMalloc/cudaFree, which take a
// device-wide lock and synchronise the device. The caller passes device pointers for the
// amplitudes and the results; the only other device memory used is the file-scope array below,
// of a fixed maximum size, which every GPU that loads the library holds until the process exits.

namespace lsg {

constexpr size_t kNoAllocScratchBytes = LSG_NOALLOC_SCRATCH_BYTES;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// The array's device address on each device. Host code must not use the symbol itself: on the
// host it names a host-side stand-in, not device memory.
static std::mutex g_noalloc_mu;
static void* g_noalloc_addr[64] = {};

static int noalloc_scratch(void** out) {
    int dev = 0;
    LSG_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return fail(LSG_E_ARG, "device %d is out of range", dev);
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
        void* ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || !ptr)
            return fail(LSG_E_CUDA, "cudaGetSymbolAddress of the scratch array failed: %s", cudaGetErrorString(e));
        g_noalloc_addr[dev] = ptr;
    }
    *out = g_noalloc_addr[dev];
    return LSG_OK;
}

// Sum each row of partials (row = member * nterms + t) in a fixed order and store it at
// out[t * batch + member], the layout lsg_expect_pauli returns.
__global__ void k_sum_rows_to_terms(const double* __restrict__ partials, int64_t ncols, int nterms, int64_t batch,
                                    double* __restrict__ out) {
    const int64_t rows = (int64_t)nterms * batch;
    for (int64_t row = blockIdx.x; row < rows; row += gridDim.x) {
        double acc = 0.0;
        for (int64_t c = threadIdx.x; c < ncols; c += blockDim.x) acc += partials[row * ncols + c];
        double tot = block_sum(acc);
        if (threadIdx.x == 0) {
            const int64_t member = row / nterms, t = row % nterms;
            out[t * batch + member] = tot;
        }
    }
}

}  // namespace lsg

extern "C" int lsg_expect_pauli_noalloc(const void* amplitudes, int precision, int nbits, int64_t batch, int dm_qubits,
                                        const uint64_t* xmask, const uint64_t* zmask, int32_t nterms,
                                        double* out_device, void* stream) {
    using namespace lsg;
    clear_error();
    if (!amplitudes || !out_device || nterms < 1 || !xmask || !zmask || batch < 1)
        return fail(LSG_E_ARG, "lsg_expect_pauli_noalloc: bad arguments");
    if (batch > kMaxGridY)
        return fail(LSG_E_ARG, "lsg_expect_pauli_noalloc: %lld members; one call takes at most %d",
                    (long long)batch, (int)kMaxGridY);
    if (precision != LSG_C128 && precision != LSG_C64) return fail(LSG_E_ARG, "unknown precision %d", precision);
    if (nbits < 0 || nbits > kMaxBits) return fail(LSG_E_CAPACITY, "a register of %d bits exceeds the engine's %d", nbits, kMaxBits);
    if (dm_qubits && 2 * dm_qubits != nbits) return fail(LSG_E_STATE, "density register size mismatch");
    const int nq = dm_qubits ? dm_qubits : nbits;
    const uint64_t limit = nq >= 64 ? ~0ull : ((1ull << nq) - 1);
    for (int t = 0; t < nterms; ++t)
        if ((xmask[t] | zmask[t]) & ~limit) return fail(LSG_E_ARG, "term %d names a missing qubit", t);
    // scratch layout: x masks | z masks | partial sums (rows x grid), each 256-byte aligned
    const size_t mask_bytes = ((size_t)nterms * 8 + 255) & ~size_t(255);
    const int64_t rows = (int64_t)nterms * batch;
    const size_t room = kNoAllocScratchBytes - 2 * std::min(mask_bytes, kNoAllocScratchBytes / 2);
    if (2 * mask_bytes >= kNoAllocScratchBytes || (size_t)rows * 8 > room)
        return fail(LSG_E_ARG,
                    "lsg_expect_pauli_noalloc: %d terms x %lld members need more than the %zu-byte scratch array "
                    "(at most %zu partial sums)", nterms, (long long)batch, kNoAllocScratchBytes, room / 8);
    const int64_t count = dm_qubits ? (1ll << dm_qubits) : (1ll << nbits);
    const int64_t fit = (int64_t)(room / 8 / (size_t)rows);
    const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>({(int64_t)reduce_grid(count), fit,
                                                                             std::max<int64_t>(1, 4096 / batch)}));
    // both buffers must be device memory of the current device: the scratch array used below is
    // the current device's, and the kernels read and write the buffers from that device
    int dev = 0;
    LSG_CUDA(cudaGetDevice(&dev));
    for (const void* ptr : {amplitudes, static_cast<const void*>(out_device)}) {
        cudaPointerAttributes attr{};
        if (cudaPointerGetAttributes(&attr, ptr) != cudaSuccess) {
            cudaGetLastError();
            return fail(LSG_E_ARG, "lsg_expect_pauli_noalloc: %s is not a CUDA pointer",
                        ptr == amplitudes ? "amplitudes" : "out_device");
        }
        const bool on_device = attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged;
        if (!on_device || attr.device != dev)
            return fail(LSG_E_ARG, "lsg_expect_pauli_noalloc: %s is not device memory of the current device %d",
                        ptr == amplitudes ? "amplitudes" : "out_device", dev);
    }
    void* base = nullptr;
    LSG_CHECK(noalloc_scratch(&base));
    char* scratch = static_cast<char*>(base);
    uint64_t* dx = reinterpret_cast<uint64_t*>(scratch);
    uint64_t* dz = reinterpret_cast<uint64_t*>(scratch + mask_bytes);
    double* part = reinterpret_cast<double*>(scratch + 2 * mask_bytes);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    LSG_CUDA(cudaMemcpyAsync(dx, xmask, (size_t)nterms * 8, cudaMemcpyHostToDevice, st));
    LSG_CUDA(cudaMemcpyAsync(dz, zmask, (size_t)nterms * 8, cudaMemcpyHostToDevice, st));
    const dim3 g2(grid, (unsigned)batch);
    const int64_t elems = 1ll << nbits;
    if (precision == LSG_C128)
        k_expect<double><<<g2, kThreads, 0, st>>>(static_cast<const Cx<double>*>(amplitudes), elems, dm_qubits, dx, dz,
                                                 nterms, part);
    else
        k_expect<float><<<g2, kThreads, 0, st>>>(static_cast<const Cx<float>*>(amplitudes), elems, dm_qubits, dx, dz,
                                                nterms, part);
    k_sum_rows_to_terms<<<(unsigned)std::min<int64_t>(rows, 152 * 16), kThreads, 0, st>>>(part, grid, nterms, batch,
                                                                                        out_device);
    LSG_CUDA(cudaGetLastError());
    // the masks are copied from the caller's host memory: wait, so the caller may reuse it
    LSG_CUDA(cudaStreamSynchronize(st));
    return LSG_OK;
}
