// Trajectory programs: Orrery's per-shot interpreter (_trajectory, simulator.py:287-317, and the
// shot loop :364-371) on the device.
//
// A program is a flattened operation list (gates, mixture and Kraus channels, measurements,
// resets, if/else markers) compiled once into steps over a register whose members are shots:
//   * runs of unitary gates and state-independent mixture channels (Pauli noise) become fused
//     tile passes; each member picks its mixture branch from its own uniform (engines.py:161-171);
//   * a measurement is a per-member FP64 p(1) reduction, a decision kernel that draws the outcome
//     (and the readout flip) from the member's uniforms, and a collapse-and-renormalise pass
//     (engines.py:185-205, simulator.py:300-306); a reset applies X after an outcome of 1;
//   * a Kraus channel is a per-member reduced density matrix, a decision by cumulative Born
//     weights (engines.py:172-183) and a per-member operator pass;
//   * if/else sets per-member predicate bits from the classical bits (circuit.py:70-72); steps in
//     a branch run only on members whose bit is set.
// Every member consumes its uniforms from a cursor in exactly the reference's order. In serial
// mode one member runs the shots one after another on one shared stream (bit-identical draws to
// Orrery); in batched mode every member is a shot with its own row of uniforms.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "program.cuh"
#include "tile.cuh"

struct lsg_program_s;

namespace lsg {

int program_create_ex(int nbits, int precision, int64_t batch, const lsg_op* ops, int32_t nops, const double* pool,
                      int64_t pool_entries, const int* pred, const int* draw, const int* count, lsg_program_s** out,
                      cudaStream_t stream);
int program_run_ctx(lsg_program_s* p, lsg_state_s* s, cudaEvent_t* marks, const TrajCtx& ctx);
void program_destroy(lsg_program_s* p);
int op_bits_ok(const lsg_op& op, int nbits);

constexpr int kT = 256;
constexpr int kMaxWords = 4;  // classical bits per shot: up to 256
constexpr double kNear = 1e-12;

enum StepKind { STEP_SEG, STEP_ADVANCE, STEP_MEASURE, STEP_KRAUS, STEP_IF };

struct Step {
    int kind = 0;
    lsg_program_s* seg = nullptr;
    int slot = 0;       // predicate bit the step runs under
    int64_t count = 0;  // ADVANCE: uniforms the segment drew
    // MEASURE / RESET
    int q = 0, clbit = -1, readout = 0, is_reset = 0;
    double p01 = 0, p10 = 0;
    // KRAUS
    int k = 0, bits[2] = {0, 0}, nkraus = 0;
    int64_t kraus_at = 0;  // offset (complex entries) in the Kraus buffer
    // IF
    int then_slot = 0, else_slot = 0, ncond = 0, negate = 0;
    uint64_t value = 0;
    int cond[64] = {};
};

__device__ __forceinline__ double nrm(double re, double im) { return re * re + im * im; }

// |a|^2 of one amplitude as a double: complex128 squares in FP64; a complex64 amplitude's square
// is formed in FP32 (exact to its own precision) and accumulated in FP64 by the caller, so the
// FP64 unit does one add per element instead of two multiply-adds.
__device__ __forceinline__ double nrm2(Cx<double> a) { return nrm(a.re, a.im); }
__device__ __forceinline__ double nrm2(Cx<float> a) { return (double)fmaf(a.re, a.re, a.im * a.im); }

__device__ double t_block_sum(double v) {
    __shared__ double buf[kT];
    buf[threadIdx.x] = v;
    __syncthreads();
    for (int s = kT / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) buf[threadIdx.x] += buf[threadIdx.x + s];
        __syncthreads();
    }
    double out = buf[0];
    __syncthreads();
    return out;
}

__device__ __forceinline__ bool has(const uint64_t* pred, int64_t b, int slot) { return (pred[b] >> slot) & 1; }

__global__ void k_t_init(uint64_t* pred, uint64_t* clbits, int64_t* cursor, int64_t batch, int words, int reset_cursor) {
    for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < batch; b += (int64_t)gridDim.x * blockDim.x) {
        pred[b] = 1;  // slot 0: the main line, always taken
        for (int w = 0; w < words; ++w) clbits[b * words + w] = 0;
        if (reset_cursor) cursor[b] = 0;
    }
}

// every member set to |0...0>
template <typename R>
__global__ void k_t_basis(Cx<R>* state, int64_t elems, int64_t total) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x)
        state[i] = Cx<R>(i % elems == 0 ? R(1) : R(0), R(0));
}

__global__ void k_t_advance(int64_t* cursor, const uint64_t* pred, int slot, int64_t count, int64_t batch) {
    for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < batch; b += (int64_t)gridDim.x * blockDim.x)
        if (has(pred, b, slot)) cursor[b] += count;
}

// per-member partial sums of |a|^2 over indices with bit q = 1; partials[b * gridDim.x + block].
// complex64 reads 16 bytes (two amplitudes) at a time.
template <typename R>
__global__ void k_t_p1(const Cx<R>* __restrict__ state, int64_t elems, int q, const uint64_t* pred, int slot,
                       double* __restrict__ partials) {
    const int64_t b = blockIdx.y;
    double acc = 0.0;
    if (has(pred, b, slot)) {
        const Cx<R>* s = state + b * elems;
        const int64_t stride = (int64_t)gridDim.x * blockDim.x;
        if constexpr (sizeof(R) == 4) {
            if (q == 0) {  // the odd amplitudes: the second half of every 16-byte pair
                for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < (elems >> 1); j += stride) {
                    const float4 w = *reinterpret_cast<const float4*>(s + 2 * j);
                    acc += nrm2(Cx<R>(w.z, w.w));
                }
            } else {  // two consecutive amplitudes with bit q set per load
                for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < (elems >> 2); j += stride) {
                    const uint64_t i = 2 * (uint64_t)j;
                    const uint64_t idx = ((i >> q) << (q + 1)) | (1ull << q) | (i & ((1ull << q) - 1));
                    const float4 w = *reinterpret_cast<const float4*>(s + idx);
                    acc += nrm2(Cx<R>(w.x, w.y)) + nrm2(Cx<R>(w.z, w.w));
                }
            }
        } else {
            const int64_t half = elems >> 1;
            for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < half; i += stride) {
                const uint64_t lo = (uint64_t)i & ((1ull << q) - 1);
                const uint64_t idx = (((uint64_t)i >> q) << (q + 1)) | (1ull << q) | lo;
                acc += nrm2(s[idx]);
            }
        }
    }
    const double tot = t_block_sum(acc);
    if (threadIdx.x == 0) partials[b * gridDim.x + blockIdx.x] = tot;
}

// one thread per member: draw the outcome (and the readout flip), record the classical bit
__global__ void k_t_decide(const double* __restrict__ partials, int nparts, int64_t* cursor, const double* __restrict__ u,
                           int64_t ustride, const uint64_t* pred, int slot, int clbit, int readout, double p01,
                           double p10, int is_reset, uint64_t* clbits, int words, int* outcome, double* prob,
                           unsigned long long* near, int64_t batch) {
    for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < batch; b += (int64_t)gridDim.x * blockDim.x) {
        if (!has(pred, b, slot)) {
            outcome[b] = -1;
            continue;
        }
        double p1 = 0.0;
        for (int g = 0; g < nparts; ++g) p1 += partials[b * nparts + g];
        p1 = fmin(fmax(p1, 0.0), 1.0);
        const double r = u[b * ustride + cursor[b]];
        cursor[b] += 1;
        if (fabs(r - p1) < kNear) atomicAdd(near, 1ull);
        int out = r < p1 ? 1 : 0;
        outcome[b] = out;
        prob[b] = out ? p1 : 1.0 - p1;
        if (!is_reset) {
            int seen = out;
            if (readout) {
                const double r2 = u[b * ustride + cursor[b]];
                cursor[b] += 1;
                if (r2 < (out ? p10 : p01)) seen ^= 1;
            }
            if (clbit >= 0) {
                uint64_t& w = clbits[b * words + (clbit >> 6)];
                const uint64_t bit = 1ull << (clbit & 63);
                w = seen ? (w | bit) : (w & ~bit);
            }
        }
    }
}

// Collapse onto the drawn outcome: the outcome's half divided by sqrt(probability), the other half
// zero (a reset with outcome 1 then applies X: the kept half moves to bit q = 0). With q_next >= 0
// the same pass accumulates the next measurement's p(1) partials over the new amplitudes, as
// k_t_p1 would (members this step skips keep their state and are summed too). complex64 moves 16
// bytes (two amplitudes) per access and reads only the half it keeps.
template <typename R>
__global__ void k_t_collapse(Cx<R>* __restrict__ state, int64_t elems, int q, const int* outcome, const double* prob,
                             int is_reset, int q_next, const uint64_t* pred, int slot_next,
                             double* __restrict__ partials) {
    const int64_t b = blockIdx.y;
    const int out = outcome[b];
    const bool want = q_next >= 0 && has(pred, b, slot_next);
    Cx<R>* s = state + b * elems;
    const double p = out >= 0 ? prob[b] : 1.0;
    const double div = p > 0 ? sqrt(p) : 1.0;
    const bool scale = out >= 0 && p > 0;
    // complex128 divides by the FP64 norm exactly as Orrery does; complex64 multiplies by its
    // FP64 reciprocal rounded once (an FP64 division per element would bind the pass to FP64)
    const R inv = (R)(1.0 / div);
    auto fix = [&](Cx<R> a) {
        if (!scale) return a;
        if constexpr (sizeof(R) == 8) return Cx<R>(a.re / div, a.im / div);
        else return Cx<R>(a.re * inv, a.im * inv);
    };
    const Cx<R> zero(R(0), R(0));
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    double acc = 0.0;
    // new amplitudes of the pair (bit q = 0, bit q = 1) from the kept one
    auto pair = [&](Cx<R> a0, Cx<R> a1, Cx<R>* n0, Cx<R>* n1) {
        if (out == 0) *n0 = fix(a0), *n1 = zero;
        else if (is_reset) *n0 = fix(a1), *n1 = zero;
        else *n0 = zero, *n1 = fix(a1);
    };
    auto count = [&](uint64_t idx, Cx<R> a) {
        if (want && ((idx >> q_next) & 1)) acc += nrm2(a);
    };
    if (out >= 0 || want) {
        if constexpr (sizeof(R) == 4) {
            if (q == 0) {  // one 16-byte load holds the pair
                for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < (elems >> 1); j += stride) {
                    const uint64_t idx = 2 * (uint64_t)j;
                    float4* at = reinterpret_cast<float4*>(s + idx);
                    const float4 w = *at;
                    Cx<R> n0(w.x, w.y), n1(w.z, w.w);
                    if (out >= 0) {
                        pair(n0, n1, &n0, &n1);
                        *at = make_float4(n0.re, n0.im, n1.re, n1.im);
                    }
                    count(idx, n0);
                    count(idx + 1, n1);
                }
            } else {  // two consecutive pairs: 16 bytes from each half
                for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < (elems >> 2); j += stride) {
                    const uint64_t i = 2 * (uint64_t)j;
                    const uint64_t i0 = ((i >> q) << (q + 1)) | (i & ((1ull << q) - 1));
                    const uint64_t i1 = i0 | (1ull << q);
                    float4* at0 = reinterpret_cast<float4*>(s + i0);
                    float4* at1 = reinterpret_cast<float4*>(s + i1);
                    Cx<R> a0, b0, a1, b1;  // (i0, i0+1), (i1, i1+1)
                    if (out < 0 || out == 0 || want) {
                        const float4 w = *at0;
                        a0 = Cx<R>(w.x, w.y), b0 = Cx<R>(w.z, w.w);
                    }
                    if (out < 0 || out == 1 || want) {
                        const float4 w = *at1;
                        a1 = Cx<R>(w.x, w.y), b1 = Cx<R>(w.z, w.w);
                    }
                    if (out >= 0) {
                        pair(a0, a1, &a0, &a1);
                        pair(b0, b1, &b0, &b1);
                        *at0 = make_float4(a0.re, a0.im, b0.re, b0.im);
                        *at1 = make_float4(a1.re, a1.im, b1.re, b1.im);
                    }
                    count(i0, a0);
                    count(i0 + 1, b0);
                    count(i1, a1);
                    count(i1 + 1, b1);
                }
            }
        } else {
            const int64_t half = elems >> 1;
            for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < half; i += stride) {
                const uint64_t lo = (uint64_t)i & ((1ull << q) - 1);
                const uint64_t i0 = (((uint64_t)i >> q) << (q + 1)) | lo;
                const uint64_t i1 = i0 | (1ull << q);
                Cx<R> n0 = s[i0], n1 = s[i1];
                if (out >= 0) {
                    pair(n0, n1, &n0, &n1);
                    s[i0] = n0;
                    s[i1] = n1;
                }
                count(i0, n0);
                count(i1, n1);
            }
        }
    }
    if (q_next >= 0) {
        const double tot = t_block_sum(acc);
        if (threadIdx.x == 0) partials[b * gridDim.x + blockIdx.x] = tot;
    }
}

// ---- consecutive measurements of distinct qubits in one group (batched mode)
//
// Measurements with nothing between them draw their outcomes from one joint distribution: one
// pass sums |a|^2 per member into the 2^g bins of the group's bits, the decisions then run in
// program order from the bins (each outcome's probability conditioned on the earlier ones, as the
// collapsed and renormalised state would give it), and one pass moves the kept slice to its final
// pattern (a reset's bit to 0) scaled to norm 1 and zeroes the rest: two passes instead of a
// reduction and a collapse per measurement.
constexpr int kGroupMax = 4;

struct Group {
    int g = 0;
    int q[kGroupMax] = {};  // register bit of measurement i (group bit i)
    int clbit[kGroupMax] = {}, readout[kGroupMax] = {}, is_reset[kGroupMax] = {};
    double p01[kGroupMax] = {}, p10[kGroupMax] = {};
};

// the group's 2^g elements around `base` (group bits 0): element k has group bit i = bit i of k
__device__ __forceinline__ uint64_t group_elem(uint64_t base, const Group& gr, int k) {
    for (int i = 0; i < gr.g; ++i) base |= (uint64_t)((k >> i) & 1) << gr.q[i];
    return base;
}

// Lanes map to (group, pattern): 2^g consecutive lanes hold the 2^g elements of one group (the
// elements that differ only in the group's bits), each lane always the same pattern, so the
// accesses of a warp are contiguous when the group's bits are the lowest ones.
__device__ __forceinline__ void sort_bits(const Group& gr, int* sorted) {
    for (int i = 0; i < gr.g; ++i) sorted[i] = gr.q[i];
    for (int i = 1; i < gr.g; ++i)  // insertion sort: spread() wants ascending positions
        for (int j = i; j > 0 && sorted[j - 1] > sorted[j]; --j) {
            const int x = sorted[j];
            sorted[j] = sorted[j - 1];
            sorted[j - 1] = x;
        }
}

constexpr int kGroupUnroll = 4;  // groups per lane per iteration: independent loads in flight

// per-member partial sums of |a|^2 per group pattern: partials[(b * gridDim.x + block) * 16 + k]
template <typename R>
__global__ void k_t_hist(const Cx<R>* __restrict__ state, int64_t elems, Group gr, const uint64_t* pred, int slot,
                         double* __restrict__ partials) {
    __shared__ double buf[kT];
    const int64_t b = blockIdx.y;
    const int k = threadIdx.x & ((1 << gr.g) - 1);
    double acc = 0.0;
    if (has(pred, b, slot)) {
        const Cx<R>* s = state + b * elems;
        int sorted[kGroupMax];
        sort_bits(gr, sorted);
        const int64_t groups = elems >> gr.g, per_block = blockDim.x >> gr.g, step = (int64_t)gridDim.x * per_block;
        const uint64_t own = group_elem(0, gr, k);  // this lane's pattern, deposited at the group's bits
        const bool low = sorted[gr.g - 1] == gr.g - 1;  // the group's bits are the lowest: base = r << g
        for (int64_t r0 = blockIdx.x * per_block + (threadIdx.x >> gr.g); r0 < groups; r0 += step * kGroupUnroll) {
            Cx<R> a[kGroupUnroll];
#pragma unroll
            for (int j = 0; j < kGroupUnroll; ++j) {
                const int64_t r = r0 + j * step;
                const uint64_t base = low ? (uint64_t)r << gr.g : spread((uint64_t)r, sorted, gr.g);
                a[j] = r < groups ? s[base | own] : Cx<R>(R(0), R(0));
            }
#pragma unroll
            for (int j = 0; j < kGroupUnroll; ++j) acc += nrm2(a[j]);
        }
    }
    buf[threadIdx.x] = acc;
    __syncthreads();
    if (threadIdx.x < (1 << gr.g)) {  // lanes of one pattern: every 2^g-th entry
        double tot = 0.0;
        for (int t = threadIdx.x; t < (int)blockDim.x; t += 1 << gr.g) tot += buf[t];
        partials[(b * gridDim.x + blockIdx.x) * (1 << kGroupMax) + threadIdx.x] = tot;
    }
}

// one thread per member: the group's outcomes in program order from the joint bins, each with its
// readout flip and classical bit as k_t_decide records them; outcome[b] = drawn pattern | final
// pattern << 8 (-1: not taken), prob[b] = the scale that renormalises the kept slice
__global__ void k_t_decide_group(const double* __restrict__ partials, int nparts, int64_t* cursor,
                                 const double* __restrict__ u, int64_t ustride, const uint64_t* pred, int slot, Group gr,
                                 uint64_t* clbits, int words, int* outcome, double* prob, unsigned long long* near,
                                 int64_t batch) {
    for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < batch; b += (int64_t)gridDim.x * blockDim.x) {
        if (!has(pred, b, slot)) {
            outcome[b] = -1;
            continue;
        }
        double bins[1 << kGroupMax];
        double total = 0.0;
        for (int k = 0; k < (1 << gr.g); ++k) {
            double v = 0.0;
            for (int p = 0; p < nparts; ++p) v += partials[((int64_t)b * nparts + p) * (1 << kGroupMax) + k];
            bins[k] = v;
            total += v;
        }
        int known = 0, val = 0, fin = 0;
        for (int i = 0; i < gr.g; ++i) {
            double num = 0.0, den = 0.0;
            for (int k = 0; k < (1 << gr.g); ++k) {
                if ((k & known) != val) continue;
                den += bins[k];
                if ((k >> i) & 1) num += bins[k];
            }
            const double p1 = den > 0.0 ? fmin(fmax(num / den, 0.0), 1.0) : 0.0;
            const double r = u[b * ustride + cursor[b]];
            cursor[b] += 1;
            if (fabs(r - p1) < kNear) atomicAdd(near, 1ull);
            const int out = r < p1 ? 1 : 0;
            known |= 1 << i;
            val |= out << i;
            if (gr.is_reset[i]) continue;  // a reset ends with its bit at 0
            fin |= out << i;
            int seen = out;
            if (gr.readout[i]) {
                const double r2 = u[b * ustride + cursor[b]];
                cursor[b] += 1;
                if (r2 < (out ? gr.p10[i] : gr.p01[i])) seen ^= 1;
            }
            if (gr.clbit[i] >= 0) {
                uint64_t& w = clbits[b * words + (gr.clbit[i] >> 6)];
                const uint64_t bit = 1ull << (gr.clbit[i] & 63);
                w = seen ? (w | bit) : (w & ~bit);
            }
        }
        outcome[b] = val | (fin << 8);
        prob[b] = bins[val] > 0.0 ? sqrt(total / bins[val]) : 1.0;
    }
}

// the group's collapse: in every group of 2^g elements the element with the final pattern takes
// the drawn pattern's amplitude times the scale and every other element becomes 0. Every lane of
// a group reads the drawn pattern's element (one address for the 2^g lanes), the warp
// synchronises, then every lane writes its own element: all lanes run the same iterations (work
// past the last group is predicated off), so the full-warp barrier is well defined.
template <typename R>
__global__ void k_t_collapse_group(Cx<R>* __restrict__ state, int64_t elems, Group gr, const int* outcome,
                                   const double* prob) {
    const int64_t b = blockIdx.y;
    const int oc = outcome[b];
    if (oc < 0) return;  // the whole block leaves: the member is not in this branch
    const int val = oc & 0xff, fin = oc >> 8;
    const double sc = prob[b];
    const R s1 = (R)sc;
    Cx<R>* s = state + b * elems;
    int sorted[kGroupMax];
    sort_bits(gr, sorted);
    const int k = threadIdx.x & ((1 << gr.g) - 1);
    const int64_t groups = elems >> gr.g, per_block = blockDim.x >> gr.g, step = (int64_t)gridDim.x * per_block;
    const int64_t first = blockIdx.x * per_block + (threadIdx.x >> gr.g);
    const int64_t iters = (groups + step * kGroupUnroll - 1) / (step * kGroupUnroll);  // the same for every lane
    const uint64_t own = group_elem(0, gr, k), src = group_elem(0, gr, val);  // at the group's bits
    const bool low = sorted[gr.g - 1] == gr.g - 1;  // the group's bits are the lowest: base = r << g
    for (int64_t it = 0; it < iters; ++it) {
        Cx<R> a[kGroupUnroll];
        uint64_t base[kGroupUnroll];
#pragma unroll
        for (int j = 0; j < kGroupUnroll; ++j) {
            const int64_t r = first + (it * kGroupUnroll + j) * step;
            base[j] = r < groups ? (low ? (uint64_t)r << gr.g : spread((uint64_t)r, sorted, gr.g)) : ~0ull;
            a[j] = base[j] != ~0ull ? s[base[j] | src] : Cx<R>(R(0), R(0));
        }
        __syncwarp();
#pragma unroll
        for (int j = 0; j < kGroupUnroll; ++j) {
            if (base[j] == ~0ull) continue;
            Cx<R> out(R(0), R(0));
            if (k == fin) {
                if constexpr (sizeof(R) == 8) out = Cx<R>(a[j].re * sc, a[j].im * sc);
                else out = Cx<R>(a[j].re * s1, a[j].im * s1);
            }
            s[base[j] | own] = out;
        }
        __syncwarp();  // the next iteration's reads come after this one's writes in every lane
    }
}

// per-member reduced density matrix of the channel's bits (k <= 2): rho[r][c] summed over the
// other bits, as 2*d*d doubles per block
template <typename R>
__global__ void k_t_rdm(const Cx<R>* __restrict__ state, int64_t elems, int k, int b0, int b1, const uint64_t* pred,
                        int slot, double* __restrict__ partials) {
    const int64_t b = blockIdx.y;
    const int d = 1 << k;
    double acc[32];
    for (int i = 0; i < 2 * d * d; ++i) acc[i] = 0.0;
    if (has(pred, b, slot)) {
        const Cx<R>* s = state + b * elems;
        const int lo = k == 1 ? b0 : min(b0, b1), hi = k == 1 ? b0 : max(b0, b1);
        const int64_t groups = elems >> k;
        for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < groups; g += (int64_t)gridDim.x * blockDim.x) {
            uint64_t base = (uint64_t)g;
            base = (((base >> lo) << (lo + 1)) | (base & ((1ull << lo) - 1)));
            if (k == 2) base = (((base >> hi) << (hi + 1)) | (base & ((1ull << hi) - 1)));
            Cx<R> v[4];
            for (int j = 0; j < d; ++j) {
                uint64_t o = 0;
                if (k == 1) o = (uint64_t)(j & 1) << b0;
                else o = ((uint64_t)((j >> 1) & 1) << b0) | ((uint64_t)(j & 1) << b1);
                v[j] = s[base | o];
            }
            for (int r = 0; r < d; ++r)
                for (int c = 0; c < d; ++c) {  // v_r conj(v_c)
                    acc[2 * (r * d + c)] += (double)v[r].re * v[c].re + (double)v[r].im * v[c].im;
                    acc[2 * (r * d + c) + 1] += (double)v[r].im * v[c].re - (double)v[r].re * v[c].im;
                }
        }
    }
    for (int i = 0; i < 2 * d * d; ++i) {
        const double tot = t_block_sum(acc[i]);
        if (threadIdx.x == 0) partials[(b * gridDim.x + blockIdx.x) * 2 * d * d + i] = tot;
    }
}

// one thread per member: Born weights Tr(K rho K^dagger) in order, pick by the member's uniform,
// write K/sqrt(w) (or the identity when no branch has weight) for the member
template <typename R>
__global__ void k_t_kraus_decide(const double* __restrict__ partials, int nparts, int k, const double* __restrict__ kraus,
                                 int nkraus, int64_t* cursor, const double* __restrict__ u, int64_t ustride,
                                 const uint64_t* pred, int slot, Cx<R>* dyn, int* apply, unsigned long long* near,
                                 int64_t batch) {
    const int d = 1 << k;
    for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < batch; b += (int64_t)gridDim.x * blockDim.x) {
        apply[b] = 0;
        if (!has(pred, b, slot)) continue;
        double rho[32];
        for (int i = 0; i < 2 * d * d; ++i) {
            double s = 0.0;
            for (int g = 0; g < nparts; ++g) s += partials[(b * nparts + g) * 2 * d * d + i];
            rho[i] = s;
        }
        const double r = u[b * ustride + cursor[b]];
        cursor[b] += 1;
        double acc = 0.0, w = 0.0;
        int pick = -1;
        for (int i = 0; i < nkraus; ++i) {
            const double* K = kraus + (int64_t)i * 2 * d * d;
            // w = sum_{r,c,c'} K[r][c] rho[c][c'] conj(K[r][c'])
            double wi = 0.0;
            for (int rr = 0; rr < d; ++rr)
                for (int c = 0; c < d; ++c)
                    for (int c2 = 0; c2 < d; ++c2) {
                        const double ar = K[2 * (rr * d + c)], ai = K[2 * (rr * d + c) + 1];
                        const double br = K[2 * (rr * d + c2)], bi = -K[2 * (rr * d + c2) + 1];
                        const double pr = rho[2 * (c * d + c2)], pi = rho[2 * (c * d + c2) + 1];
                        // Re(a * p * b)
                        const double apr = ar * pr - ai * pi, api = ar * pi + ai * pr;
                        wi += apr * br - api * bi;
                    }
            w = wi;
            acc += wi;
            if (fabs(r - acc) < kNear) atomicAdd(near, 1ull);
            if (r < acc && wi > 0) {
                pick = i;
                break;
            }
        }
        if (pick < 0) pick = nkraus - 1;  // nothing chosen: the last candidate (engines.py:181-183)
        Cx<R>* m = dyn + b * d * d;
        if (w > 0) {
            const double sc = sqrt(w);
            const double* K = kraus + (int64_t)pick * 2 * d * d;
            for (int i = 0; i < d * d; ++i) m[i] = Cx<R>((R)(K[2 * i] / sc), (R)(K[2 * i + 1] / sc));
            apply[b] = 1;
        }
    }
}

// per-member dense operator on k <= 2 bits (b0 = most significant)
template <typename R>
__global__ void k_t_apply_dyn(Cx<R>* __restrict__ state, int64_t elems, int k, int b0, int b1, const Cx<R>* dyn,
                              const int* apply) {
    const int64_t b = blockIdx.y;
    if (!apply[b]) return;
    const int d = 1 << k;
    Cx<R>* s = state + b * elems;
    const Cx<R>* m = dyn + b * d * d;
    const int lo = k == 1 ? b0 : min(b0, b1), hi = k == 1 ? b0 : max(b0, b1);
    const int64_t groups = elems >> k;
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < groups; g += (int64_t)gridDim.x * blockDim.x) {
        uint64_t base = (uint64_t)g;
        base = (((base >> lo) << (lo + 1)) | (base & ((1ull << lo) - 1)));
        if (k == 2) base = (((base >> hi) << (hi + 1)) | (base & ((1ull << hi) - 1)));
        uint64_t offs[4];
        Cx<R> v[4];
        for (int j = 0; j < d; ++j) {
            offs[j] = k == 1 ? ((uint64_t)(j & 1) << b0) : (((uint64_t)((j >> 1) & 1) << b0) | ((uint64_t)(j & 1) << b1));
            v[j] = s[base | offs[j]];
        }
        for (int r = 0; r < d; ++r) {
            Cx<R> acc;
            for (int c = 0; c < d; ++c) acc = cfma(m[r * d + c], v[c], acc);
            s[base | offs[r]] = acc;
        }
    }
}

struct Cond {
    int n, negate;
    uint64_t value;
    int bits[64];
};

__global__ void k_t_if(uint64_t* pred, const uint64_t* clbits, int words, int parent, int then_slot, int else_slot,
                       Cond c, int64_t batch) {
    for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < batch; b += (int64_t)gridDim.x * blockDim.x) {
        uint64_t p = pred[b] & ~((1ull << then_slot) | (1ull << else_slot));
        if ((p >> parent) & 1) {
            uint64_t reading = 0;
            for (int i = 0; i < c.n; ++i) {
                const int cb = c.bits[i];
                reading |= ((clbits[b * words + (cb >> 6)] >> (cb & 63)) & 1ull) << i;
            }
            const bool holds = (reading == c.value) != (c.negate != 0);
            p |= holds ? (1ull << then_slot) : (1ull << else_slot);
        }
        pred[b] = p;
    }
}

__global__ void k_t_record(const uint64_t* clbits, int words, uint64_t* out, int64_t* shot) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        const int64_t s = *shot;
        for (int w = 0; w < words; ++w) out[s * words + w] = clbits[w];
        *shot = s + 1;
    }
}

unsigned t_grid(int64_t n) { return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + kT - 1) / kT, 152 * 16)); }

}  // namespace lsg

using namespace lsg;

struct lsg_traj_s {
    int nbits = 0, precision = 0, words = 1;
    int64_t batch = 1;
    int64_t max_draws = 0;
    std::vector<Step> steps;
    Scratch kraus;  // all Kraus matrices, complex128
    // per-run device buffers
    Scratch ctl;    // cursor, pred, clbits, outcome, prob, apply, counters
    Scratch parts;  // reduction partials
    Scratch dyn;    // per-member Kraus operators
    Scratch ubuf;   // uniforms
    Scratch results;
    ~lsg_traj_s() {
        for (Step& s : steps)
            if (s.seg) program_destroy(s.seg);
        release(kraus);
        release(ctl);
        release(parts);
        release(dyn);
        release(ubuf);
        release(results);
    }
};

namespace {

struct Ctl {
    int64_t* cursor;
    uint64_t* pred;
    uint64_t* clbits;
    int* outcome;
    double* prob;
    int* apply;
    unsigned long long* near;
    int64_t* shot;
};

int ctl_setup(lsg_traj_s* t, int64_t batch, Ctl* c) {
    auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
    const size_t need = al(batch * 8) * 2 + al(batch * 8 * t->words) + al(batch * 4) + al(batch * 8) + al(batch * 4) + 512;
    LSG_CHECK(ensure(t->ctl, need));
    char* p = (char*)t->ctl.ptr;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        char* at = p + off;
        off += al(bytes);
        return at;
    };
    c->cursor = (int64_t*)take(batch * 8);
    c->pred = (uint64_t*)take(batch * 8);
    c->clbits = (uint64_t*)take(batch * 8 * t->words);
    c->outcome = (int*)take(batch * 4);
    c->prob = (double*)take(batch * 8);
    c->apply = (int*)take(batch * 4);
    c->near = (unsigned long long*)take(8);
    c->shot = (int64_t*)take(8);
    const int dmax = 4;
    LSG_CHECK(ensure(t->dyn, (size_t)batch * dmax * dmax * 16));
    return LSG_OK;
}

// How many measurements from step `si` on form one group: consecutive, under the same predicate,
// of distinct qubits, at most kGroupMax.
int group_length(const std::vector<Step>& steps, size_t si) {
    int n = 0;
    uint64_t seen = 0;
    for (size_t j = si; j < steps.size() && n < kGroupMax; ++j, ++n) {
        const Step& m = steps[j];
        if (m.kind != STEP_MEASURE || m.slot != steps[si].slot || ((seen >> m.q) & 1)) break;
        seen |= 1ull << m.q;
    }
    return std::max(n, 1);
}

template <typename R>
int run_steps(lsg_traj_s* t, lsg_state_s* s, const Ctl& c, const double* u, int64_t ustride) {
    const int64_t B = s->batch;
    const int64_t elems = s->elems;
    cudaStream_t st = s->stream;
    Cx<R>* state = (Cx<R>*)s->data;
    TrajCtx ctx;
    ctx.u = u;
    ctx.ustride = ustride;
    ctx.cursor = c.cursor;
    ctx.pred = c.pred;
    const unsigned gx = (unsigned)std::max<int64_t>(1, std::min<int64_t>(((elems >> 1) + kT * 4 - 1) / (kT * 4),
                                                                          std::max<int64_t>(1, 8192 / B)));
    bool p1_ready = false;  // the current step's p(1) partials were accumulated by the previous collapse
    for (size_t si = 0; si < t->steps.size(); ++si) {
        const Step& sp = t->steps[si];
        bool next_p1_ready = false;
        switch (sp.kind) {
            case STEP_SEG: LSG_CHECK(program_run_ctx(sp.seg, s, nullptr, ctx)); break;
            case STEP_ADVANCE:
                k_t_advance<<<t_grid(B), kT, 0, st>>>(c.cursor, c.pred, sp.slot, sp.count, B);
                break;
            case STEP_MEASURE: {
                double* part = (double*)t->parts.ptr;
                const int glen = B > 1 ? group_length(t->steps, si) : 1;
                if (glen > 1) {  // this measurement and the next glen-1 as one group
                    Group gr;
                    gr.g = glen;
                    for (int i = 0; i < glen; ++i) {
                        const Step& m = t->steps[si + i];
                        gr.q[i] = m.q;
                        gr.clbit[i] = m.is_reset ? -1 : m.clbit;
                        gr.readout[i] = m.is_reset ? 0 : m.readout;
                        gr.is_reset[i] = m.is_reset;
                        gr.p01[i] = m.p01;
                        gr.p10[i] = m.p10;
                    }
                    k_t_hist<R><<<dim3(gx, (unsigned)B), kT, 0, st>>>(state, elems, gr, c.pred, sp.slot, part);
                    k_t_decide_group<<<t_grid(B), kT, 0, st>>>(part, (int)gx, c.cursor, u, ustride, c.pred, sp.slot, gr,
                                                              c.clbits, t->words, c.outcome, c.prob, c.near, B);
                    k_t_collapse_group<R><<<dim3(gx, (unsigned)B), kT, 0, st>>>(state, elems, gr, c.outcome, c.prob);
                    si += glen - 1;
                    break;
                }
                if (!p1_ready)
                    k_t_p1<R><<<dim3(gx, (unsigned)B), kT, 0, st>>>(state, elems, sp.q, c.pred, sp.slot, part);
                k_t_decide<<<t_grid(B), kT, 0, st>>>(part, (int)gx, c.cursor, u, ustride, c.pred, sp.slot, sp.clbit,
                                                    sp.readout, sp.p01, sp.p10, sp.is_reset, c.clbits, t->words,
                                                    c.outcome, c.prob, c.near, B);
                // a measurement right after this one: its p(1) partials come out of this collapse
                const Step* nx = si + 1 < t->steps.size() ? &t->steps[si + 1] : nullptr;
                const bool fuse = nx && nx->kind == STEP_MEASURE && (B == 1 || group_length(t->steps, si + 1) == 1);
                k_t_collapse<R><<<dim3(gx, (unsigned)B), kT, 0, st>>>(state, elems, sp.q, c.outcome, c.prob, sp.is_reset,
                                                                    fuse ? nx->q : -1, c.pred, fuse ? nx->slot : 0, part);
                next_p1_ready = fuse;
                break;
            }
            case STEP_KRAUS: {
                double* part = (double*)t->parts.ptr;
                k_t_rdm<R><<<dim3(gx, (unsigned)B), kT, 0, st>>>(state, elems, sp.k, sp.bits[0], sp.bits[1], c.pred,
                                                               sp.slot, part);
                k_t_kraus_decide<R><<<t_grid(B), kT, 0, st>>>(part, (int)gx, sp.k, (const double*)t->kraus.ptr + 2 * sp.kraus_at,
                                                             sp.nkraus, c.cursor, u, ustride, c.pred, sp.slot,
                                                             (Cx<R>*)t->dyn.ptr, c.apply, c.near, B);
                k_t_apply_dyn<R><<<dim3(gx, (unsigned)B), kT, 0, st>>>(state, elems, sp.k, sp.bits[0], sp.bits[1],
                                                                     (const Cx<R>*)t->dyn.ptr, c.apply);
                break;
            }
            case STEP_IF: {
                Cond cd{};
                cd.n = sp.ncond;
                cd.negate = sp.negate;
                cd.value = sp.value;
                for (int i = 0; i < sp.ncond; ++i) cd.bits[i] = sp.cond[i];
                k_t_if<<<t_grid(B), kT, 0, st>>>(c.pred, c.clbits, t->words, sp.slot, sp.then_slot, sp.else_slot, cd, B);
                break;
            }
            default: break;
        }
        p1_ready = next_p1_ready;
    }
    LSG_CUDA(cudaGetLastError());
    return LSG_OK;
}

int parts_setup(lsg_traj_s* t, int64_t batch, int64_t elems) {
    const int64_t gx = std::max<int64_t>(1, std::min<int64_t>(((elems >> 1) + kT * 4 - 1) / (kT * 4),
                                                              std::max<int64_t>(1, 8192 / batch)));
    return ensure(t->parts, (size_t)(batch * gx * 32 + 64) * 8);
}

}  // namespace

extern "C" {

int lsg_traj_create(lsg_state shape, const lsg_traj_op* ops, int32_t nops, const double* pool, int64_t pool_entries,
                    int32_t num_clbits, lsg_traj* out) {
    clear_error();
    if (!shape || !out || nops < 0 || (nops && !ops) || pool_entries < 0 || (pool_entries && !pool))
        return fail(LSG_E_ARG, "lsg_traj_create: bad arguments");
    *out = nullptr;
    if (shape->real()) return fail(LSG_E_ARG, "trajectories run on statevector registers");
    if (num_clbits < 0 || num_clbits > 64 * kMaxWords)
        return fail(LSG_E_CAPACITY, "trajectories on the device keep at most %d classical bits", 64 * kMaxWords);
    const int nbits = shape->nbits;
    auto* t = new lsg_traj_s();
    t->nbits = nbits;
    t->precision = shape->precision;
    t->batch = shape->batch;
    t->words = std::max(1, (num_clbits + 63) / 64);
    std::vector<double> kraus_host;
    // segment under construction
    std::vector<lsg_op> seg_ops;
    std::vector<int> seg_pred, seg_draw, seg_count;
    int seg_slot = -1;
    int64_t seg_draws = 0;
    struct Frame {
        int parent, then_slot, else_slot;
        int64_t draws_before, then_draws;
    };
    std::vector<Frame> stack;
    int slot = 0;
    int64_t draws = 0;  // upper bound along the current path
    auto fail_out = [&](int code) {
        delete t;
        return code;
    };
    auto flush = [&]() -> int {
        if (seg_ops.empty()) return LSG_OK;
        Step sp;
        sp.kind = STEP_SEG;
        sp.slot = seg_slot;
        int rc = program_create_ex(nbits, shape->precision, shape->batch, seg_ops.data(), (int32_t)seg_ops.size(), pool,
                                   pool_entries, seg_pred.data(), seg_draw.data(), seg_count.data(), &sp.seg,
                                   shape->stream);
        if (rc != LSG_OK) return rc;
        t->steps.push_back(sp);
        if (seg_draws) {
            Step adv;
            adv.kind = STEP_ADVANCE;
            adv.slot = seg_slot;
            adv.count = seg_draws;
            t->steps.push_back(adv);
        }
        seg_ops.clear();
        seg_pred.clear();
        seg_draw.clear();
        seg_count.clear();
        seg_draws = 0;
        seg_slot = -1;
        return LSG_OK;
    };
    for (int i = 0; i < nops; ++i) {
        const lsg_traj_op& op = ops[i];
        const bool unitary = op.kind == LSG_T_GATE || op.kind == LSG_T_MIXTURE || op.kind == LSG_T_SCALE;
        if (unitary) {
            if (seg_slot != slot) {
                int rc = flush();
                if (rc != LSG_OK) return fail_out(rc);
                seg_slot = slot;
            }
            lsg_op o{};
            o.nbits = op.kind == LSG_T_SCALE ? 0 : op.nq;
            for (int j = 0; j < o.nbits; ++j) o.bits[j] = op.qubits[j];
            o.data = op.data;
            o.kind = op.kind == LSG_T_GATE ? op.opkind : (op.kind == LSG_T_SCALE ? LSG_OP_SCALE : kOpMixture);
            if (!op_bits_ok(o, nbits) || (op.kind == LSG_T_MIXTURE && (op.count < 1 || op.nq > 2)))
                return fail_out(fail(LSG_E_ARG, "trajectory op %d has a bad kind or qubits", i));
            const int64_t d = 1ll << o.nbits;
            int64_t need = 1;
            if (o.kind == LSG_OP_MATRIX) need = d * d;
            else if (o.kind == LSG_OP_DIAG) need = d;
            else if (o.kind == LSG_OP_PERM) need = 2 * d;
            else if (o.kind == kOpMixture) need = op.count + op.count * d * d;
            if (op.data < 0 || op.data + need > pool_entries)
                return fail_out(fail(LSG_E_ARG, "trajectory op %d reads outside the pool", i));
            seg_ops.push_back(o);
            seg_pred.push_back(slot);
            seg_draw.push_back(op.kind == LSG_T_MIXTURE ? (int)seg_draws : 0);
            seg_count.push_back(op.kind == LSG_T_MIXTURE ? op.count : 0);
            if (op.kind == LSG_T_MIXTURE) {
                ++seg_draws;
                ++draws;
            }
            continue;
        }
        int rc = flush();
        if (rc != LSG_OK) return fail_out(rc);
        Step sp;
        sp.slot = slot;
        switch (op.kind) {
            case LSG_T_MEASURE:
            case LSG_T_RESET:
                if (op.qubits[0] < 0 || op.qubits[0] >= nbits) return fail_out(fail(LSG_E_ARG, "op %d: bad qubit", i));
                if (op.kind == LSG_T_MEASURE && op.clbit >= num_clbits)
                    return fail_out(fail(LSG_E_ARG, "op %d: bad classical bit", i));
                sp.kind = STEP_MEASURE;
                sp.q = op.qubits[0];
                sp.is_reset = op.kind == LSG_T_RESET;
                sp.clbit = op.kind == LSG_T_MEASURE ? op.clbit : -1;
                sp.readout = op.kind == LSG_T_MEASURE && op.readout;
                sp.p01 = op.p01;
                sp.p10 = op.p10;
                draws += 1 + sp.readout;
                t->steps.push_back(sp);
                break;
            case LSG_T_KRAUS: {
                if (op.nq < 1 || op.nq > 2 || op.count < 1) return fail_out(fail(LSG_E_ARG, "op %d: bad Kraus channel", i));
                const int64_t d = 1ll << op.nq;
                if (op.data < 0 || op.data + op.count * d * d > pool_entries)
                    return fail_out(fail(LSG_E_ARG, "op %d reads outside the pool", i));
                for (int j = 0; j < op.nq; ++j)
                    if (op.qubits[j] < 0 || op.qubits[j] >= nbits) return fail_out(fail(LSG_E_ARG, "op %d: bad qubit", i));
                sp.kind = STEP_KRAUS;
                sp.k = op.nq;
                sp.bits[0] = op.qubits[0];
                sp.bits[1] = op.nq > 1 ? op.qubits[1] : 0;
                sp.nkraus = op.count;
                sp.kraus_at = (int64_t)kraus_host.size() / 2;
                kraus_host.insert(kraus_host.end(), pool + 2 * op.data, pool + 2 * (op.data + op.count * d * d));
                draws += 1;
                t->steps.push_back(sp);
                break;
            }
            case LSG_T_IF: {
                const int depth = (int)stack.size();
                if (2 * depth + 2 > 63) return fail_out(fail(LSG_E_CAPACITY, "if/else nested deeper than 31 levels"));
                if (op.count < 1 || op.count > 64 || op.data < 0 || op.data + op.count > pool_entries)
                    return fail_out(fail(LSG_E_ARG, "op %d: bad condition", i));
                sp.kind = STEP_IF;
                sp.then_slot = 2 * depth + 1;
                sp.else_slot = 2 * depth + 2;
                sp.ncond = op.count;
                sp.negate = op.negate;
                sp.value = op.value;
                for (int j = 0; j < op.count; ++j) {
                    const double cb = pool[2 * (op.data + j)];
                    if (!(cb >= 0 && cb < num_clbits)) return fail_out(fail(LSG_E_ARG, "op %d: bad condition bit", i));
                    sp.cond[j] = (int)cb;
                }
                t->steps.push_back(sp);
                stack.push_back(Frame{slot, sp.then_slot, sp.else_slot, draws, 0});
                slot = sp.then_slot;
                break;
            }
            case LSG_T_ELSE:
                if (stack.empty()) return fail_out(fail(LSG_E_ARG, "op %d: else without if", i));
                stack.back().then_draws = draws - stack.back().draws_before;
                draws = stack.back().draws_before;
                slot = stack.back().else_slot;
                break;
            case LSG_T_ENDIF: {
                if (stack.empty()) return fail_out(fail(LSG_E_ARG, "op %d: endif without if", i));
                Frame f = stack.back();
                stack.pop_back();
                const int64_t branch = draws - f.draws_before;
                const int64_t taken = slot == f.then_slot ? branch : std::max(branch, f.then_draws);
                draws = f.draws_before + taken;
                slot = f.parent;
                break;
            }
            default: return fail_out(fail(LSG_E_ARG, "op %d: unknown kind %d", i, op.kind));
        }
    }
    if (!stack.empty()) return fail_out(fail(LSG_E_ARG, "an if block is not closed"));
    int rc = flush();
    if (rc != LSG_OK) return fail_out(rc);
    t->max_draws = draws;
    if (!kraus_host.empty()) {
        rc = ensure(t->kraus, kraus_host.size() * 8);
        if (rc != LSG_OK) return fail_out(rc);
        cudaError_t e = cudaMemcpy(t->kraus.ptr, kraus_host.data(), kraus_host.size() * 8, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return fail_out(fail(LSG_E_CUDA, "uploading Kraus operators failed: %s", cudaGetErrorString(e)));
    }
    *out = t;
    return LSG_OK;
}

int lsg_traj_info(lsg_traj t, int64_t* max_draws, int32_t* steps) {
    clear_error();
    if (!t) return fail(LSG_E_ARG, "null program");
    if (max_draws) *max_draws = t->max_draws;
    if (steps) *steps = (int32_t)t->steps.size();
    return LSG_OK;
}

int lsg_traj_free(lsg_traj t) {
    clear_error();
    delete t;
    return LSG_OK;
}

int lsg_traj_run_batched(lsg_traj t, lsg_state s, const double* uniforms, int64_t ustride, uint64_t* clbits_out,
                         int64_t* consumed, int64_t* near_count) {
    clear_error();
    if (!t || !s || !uniforms || !clbits_out) return fail(LSG_E_ARG, "lsg_traj_run_batched: bad arguments");
    if (s->nbits != t->nbits || s->precision != t->precision || s->batch != t->batch)
        return fail(LSG_E_STATE, "the trajectory program was built for another register shape");
    if (ustride < t->max_draws || ustride < 1)
        return fail(LSG_E_ARG, "each shot needs %lld uniforms; the stride is %lld", (long long)t->max_draws, (long long)ustride);
    const int64_t B = s->batch;
    Ctl c{};
    LSG_CHECK(ctl_setup(t, B, &c));
    LSG_CHECK(parts_setup(t, B, s->elems));
    LSG_CHECK(ensure(t->ubuf, (size_t)(B * ustride) * 8));
    LSG_CUDA(cudaMemcpyAsync(t->ubuf.ptr, uniforms, (size_t)(B * ustride) * 8, cudaMemcpyHostToDevice, s->stream));
    LSG_CUDA(cudaMemsetAsync(c.near, 0, 8, s->stream));
    const int64_t n = s->elems * B;
    if (s->precision == LSG_C128)
        k_t_basis<double><<<t_grid(n), kT, 0, s->stream>>>((Cx<double>*)s->data, s->elems, n);
    else
        k_t_basis<float><<<t_grid(n), kT, 0, s->stream>>>((Cx<float>*)s->data, s->elems, n);
    k_t_init<<<t_grid(B), kT, 0, s->stream>>>(c.pred, c.clbits, c.cursor, B, t->words, 1);
    LSG_CUDA(cudaGetLastError());
    int rc = s->precision == LSG_C128 ? run_steps<double>(t, s, c, (const double*)t->ubuf.ptr, ustride)
                                      : run_steps<float>(t, s, c, (const double*)t->ubuf.ptr, ustride);
    LSG_CHECK(rc);
    LSG_CUDA(cudaMemcpyAsync(clbits_out, c.clbits, (size_t)B * t->words * 8, cudaMemcpyDeviceToHost, s->stream));
    if (consumed) LSG_CUDA(cudaMemcpyAsync(consumed, c.cursor, (size_t)B * 8, cudaMemcpyDeviceToHost, s->stream));
    unsigned long long nr = 0;
    LSG_CUDA(cudaMemcpyAsync(&nr, c.near, 8, cudaMemcpyDeviceToHost, s->stream));
    LSG_CUDA(cudaStreamSynchronize(s->stream));
    if (near_count) *near_count = (int64_t)nr;
    return check_device_status(s->stream);
}

int lsg_traj_run_serial(lsg_traj t, lsg_state s, int64_t shots, const double* uniforms, int64_t nuniforms,
                        uint64_t* clbits_out, int64_t* consumed, int64_t* near_count) {
    clear_error();
    if (!t || !s || shots < 0 || (shots && (!uniforms || !clbits_out))) return fail(LSG_E_ARG, "lsg_traj_run_serial: bad arguments");
    if (s->nbits != t->nbits || s->precision != t->precision || s->batch != 1 || t->batch != 1)
        return fail(LSG_E_STATE, "serial trajectories run on a one-member register of the program's shape");
    if (shots == 0) {
        if (consumed) *consumed = 0;
        if (near_count) *near_count = 0;
        return LSG_OK;
    }
    if (nuniforms < shots * std::max<int64_t>(t->max_draws, 1))
        return fail(LSG_E_ARG, "%lld shots need up to %lld uniforms; %lld given", (long long)shots,
                    (long long)(shots * t->max_draws), (long long)nuniforms);
    Ctl c{};
    LSG_CHECK(ctl_setup(t, 1, &c));
    LSG_CHECK(parts_setup(t, 1, s->elems));
    LSG_CHECK(ensure(t->ubuf, (size_t)nuniforms * 8));
    LSG_CHECK(ensure(t->results, (size_t)shots * t->words * 8));
    if (!device_status()) return fail(LSG_E_CUDA, "cannot allocate the device status word");
    LSG_CUDA(cudaMemcpyAsync(t->ubuf.ptr, uniforms, (size_t)nuniforms * 8, cudaMemcpyHostToDevice, s->stream));
    LSG_CUDA(cudaMemsetAsync(c.near, 0, 8, s->stream));
    LSG_CUDA(cudaMemsetAsync(c.shot, 0, 8, s->stream));
    LSG_CUDA(cudaMemsetAsync(c.cursor, 0, 8, s->stream));
    const double* u = (const double*)t->ubuf.ptr;
    auto one_shot = [&]() -> int {
        if (s->precision == LSG_C128)
            k_t_basis<double><<<t_grid(s->elems), kT, 0, s->stream>>>((Cx<double>*)s->data, s->elems, s->elems);
        else
            k_t_basis<float><<<t_grid(s->elems), kT, 0, s->stream>>>((Cx<float>*)s->data, s->elems, s->elems);
        k_t_init<<<1, 32, 0, s->stream>>>(c.pred, c.clbits, c.cursor, 1, t->words, 0);
        int rc = s->precision == LSG_C128 ? run_steps<double>(t, s, c, u, 0) : run_steps<float>(t, s, c, u, 0);
        if (rc != LSG_OK) return rc;
        k_t_record<<<1, 32, 0, s->stream>>>(c.clbits, t->words, (uint64_t*)t->results.ptr, c.shot);
        LSG_CUDA(cudaGetLastError());
        return LSG_OK;
    };
    // one shot's launches captured once as a CUDA graph, replayed per shot
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    bool graphed = false;
    if (shots > 1 && cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
        int rc = one_shot();
        cudaError_t e = cudaStreamEndCapture(s->stream, &graph);
        if (rc == LSG_OK && e == cudaSuccess && graph &&
            cudaGraphInstantiate(&exec, graph, 0) == cudaSuccess)
            graphed = true;
        cudaGetLastError();
    }
    for (int64_t i = 0; i < shots; ++i) {
        if (graphed) {
            cudaError_t e = cudaGraphLaunch(exec, s->stream);
            if (e != cudaSuccess) {
                cudaGraphExecDestroy(exec);
                cudaGraphDestroy(graph);
                return fail(LSG_E_CUDA, "cudaGraphLaunch failed: %s", cudaGetErrorString(e));
            }
        } else {
            LSG_CHECK(one_shot());
        }
    }
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    LSG_CUDA(cudaMemcpyAsync(clbits_out, t->results.ptr, (size_t)shots * t->words * 8, cudaMemcpyDeviceToHost, s->stream));
    if (consumed) LSG_CUDA(cudaMemcpyAsync(consumed, c.cursor, 8, cudaMemcpyDeviceToHost, s->stream));
    unsigned long long nr = 0;
    LSG_CUDA(cudaMemcpyAsync(&nr, c.near, 8, cudaMemcpyDeviceToHost, s->stream));
    LSG_CUDA(cudaStreamSynchronize(s->stream));
    if (near_count) *near_count = (int64_t)nr;
    return check_device_status(s->stream);
}

}  // extern "C"
