/*
 * lsg.h — C ABI of the GB300 engine for Orrery's simulation hot path.
 *
 * Plain C types only: opaque handles, pointers and sizes. Every call returns LSG_OK (0) or a
 * negative LSG_E* code; lsg_last_error() gives the message of the calling thread's last failure.
 * The library never aborts and never throws across this boundary. Host buffers are owned by the
 * caller and never retained after a call returns. Device memory belongs to the handle.
 *
 * Index convention (Orrery, src/lucivant_sim/engines.py:8-9): amplitudes are little-endian, bit q
 * of an index is qubit q. A density matrix on n qubits is a register of 2n bits holding the
 * row-major (2^n, 2^n) matrix, so qubit q is column bit q and row bit n+q
 * (src/lucivant_sim/engines.py:222-231). A k-bit operator's index has bits[0] as its most
 * significant bit (src/lucivant_sim/gates.py:1-7).
 */
#ifndef LSG_H
#define LSG_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define LSG_OK 0
#define LSG_E_ARG (-1)       /* bad argument (maps to ValueError) */
#define LSG_E_CAPACITY (-2)  /* too large for the engine (maps to SimulationError) */
#define LSG_E_MEMORY (-3)    /* device allocation failed (maps to MemoryError) */
#define LSG_E_CUDA (-4)      /* a CUDA call failed */
#define LSG_E_TIMEOUT (-5)   /* a bounded device wait gave up; the result is not valid */
#define LSG_E_STATE (-6)     /* the call does not fit the handle (wrong kind or size) */

/* precisions */
#define LSG_C128 0 /* complex128 amplitudes, FP64 arithmetic */
#define LSG_C64 1  /* complex64 amplitudes, FP32 arithmetic; reductions stay FP64 */
/* Real registers hold density matrices in Pauli-transfer form: a register of 2n bits holds the
 * 4^n real coefficients r_P = Tr(P rho) of an n-qubit density matrix, qubit q's Pauli digit in
 * register bits (n+q, q) = (x, z): I = (0,0), Z = (0,1), X = (1,0), Y = (1,1). Channels act on
 * them as real matrices (Pauli transfer matrices) through the same operator kinds (MATRIX, DIAG,
 * PERM, SCALE; pool entries must be real). Reductions with dm_qubits = n read them as the density
 * matrix they stand for. */
#define LSG_R64 2 /* real FP64 coefficients */
#define LSG_R32 3 /* real FP32 coefficients; reductions stay FP64 */
#define LSG_RD 4  /* real coefficients as double-float pairs (hi + lo, two FP32 words, 8 bytes): about
                           48 significant bits from FP32 arithmetic; reductions in FP64 */

/* operator kinds for lsg_apply */
#define LSG_OP_MATRIX 0 /* dense 2^k x 2^k complex matrix, row-major, on bits[0..k), k <= 5 */
#define LSG_OP_DIAG 1   /* 2^k complex diagonal entries */
#define LSG_OP_PERM 2   /* out[r] = phase[r] * in[src[r]]: 2^k complex phases, then 2^k sources (real
                           part), k <= 5 */
#define LSG_OP_DEPOL 3  /* (1-p) rho + (p/d) I (x) Tr_t rho on a density register: bits = k row bits then
                           k column bits; data holds p in its real part */
#define LSG_OP_SCALE 4  /* multiply every amplitude by one complex factor (a global phase) */

#define LSG_MAX_OP_BITS 8

typedef struct lsg_op {
    int32_t kind;
    int32_t nbits;                 /* bits the operator touches (0 for SCALE) */
    int32_t bits[LSG_MAX_OP_BITS]; /* register bit positions, most significant first */
    int64_t data;                  /* offset of the operator's data in the pool, in complex entries */
    int64_t batch_stride;          /* complex entries between batch members' data; 0 = shared */
} lsg_op;

typedef struct lsg_state_s* lsg_state;

/* ---- library ------------------------------------------------------------------------------ */
const char* lsg_last_error(void);
int lsg_version(void);
/* Bind the calling thread's calls to a device (default 0). */
int lsg_init(int device);
/* Largest register a state handle accepts, in bits (26: 2^26 amplitudes). */
int lsg_max_bits(void);
/* Free and total device memory of the calling thread's device (admission control). */
int lsg_mem_info(int64_t* free_bytes, int64_t* total_bytes);

/* ---- registers ------------------------------------------------------------------------------
 * A register holds `batch` independent members of 2^nbits amplitudes each, contiguous in HBM.
 * Replaces Statevector.__init__ / DensityMatrix.__init__ (src/lucivant_sim/engines.py:139-148,
 * :216-225); the member count is the batching axis (shots, noise instances). */
int lsg_state_create(int nbits, int precision, int64_t batch, lsg_state* out);
int lsg_state_free(lsg_state s);
/* Every member set to the basis state |index>. */
int lsg_state_set_basis(lsg_state s, int64_t index);
/* Copy all members in / out as complex128 (converted when the register is complex64), or as
 * float64 for a real register. A real register's basis state `index` is |index><index| of its
 * nbits/2 qubits, in Pauli-transfer form. */
int lsg_state_upload(lsg_state s, const double* host_c128, int64_t nbytes);
int lsg_state_download(lsg_state s, double* host_c128, int64_t nbytes);
/* Member `member` of a real (Pauli-transfer) register copied into member 0 of a complex register
 * of the same bits, as real amplitudes: applying the per-qubit change of basis to the complex
 * register then yields the density matrix. Not in Orrery (its density matrices are complex). */
int lsg_state_to_complex(lsg_state src, int64_t member, lsg_state dst);
/* Bytes of device memory the handle holds. */
int lsg_state_bytes(lsg_state s, int64_t* out);

/* ---- gate passes ----------------------------------------------------------------------------
 * Apply `nops` operators in order. The engine plans them into fused tile passes (each pass
 * loads tiles of the register into shared memory once, applies every operator of the pass and
 * writes back once). Replaces _apply_slices / _apply (src/lucivant_sim/engines.py:38-119), the
 * density-matrix gate and channel updates (:233-255, _depolarizing_trace :122-135) and the
 * static loop of _evolve (src/lucivant_sim/simulator.py:229-251). `pool` holds complex128 data as
 * (re, im) pairs; complex64 registers round it once. */
int lsg_apply(lsg_state s, const lsg_op* ops, int32_t nops, const double* pool, int64_t pool_entries);
/* lsg_state_set_basis(s, index) then lsg_apply, in one call that skips tiles the operators have not
 * reached yet (still zero; see lsg_program_run_from_basis): the evolution from |index> of
 * Statevector(n) / DensityMatrix(n) (engines.py:139-148, :216-225). */
int lsg_apply_from_basis(lsg_state s, int64_t index, const lsg_op* ops, int32_t nops, const double* pool,
                         int64_t pool_entries);

/* ---- programs: planned, uploaded operator lists ---------------------------------------------
 * lsg_program_create plans and uploads `ops` once for registers shaped like `shape` (same bits,
 * precision and batch); lsg_program_run then enqueues the passes on the register's stream without
 * any host synchronisation, so a circuit template is launched repeatedly (and can be captured
 * in a CUDA graph) at kernel-launch cost. The complex64 pool is rounded once at creation. */
typedef struct lsg_program_s* lsg_program;
int lsg_program_create(lsg_state shape, const lsg_op* ops, int32_t nops, const double* pool,
                       int64_t pool_entries, lsg_program* out);
int lsg_program_run(lsg_program p, lsg_state s);
/* Run once with CUDA events around every pass (on the register's stream) and wait: pass_ms gets
 * one device time per pass, in milliseconds. */
int lsg_program_run_timed(lsg_program p, lsg_state s, float* pass_ms);
/* Set every member to basis state `index` (as lsg_state_set_basis) and run the program from it,
 * visiting only tiles that can be nonzero: register bits no earlier non-diagonal operator has
 * touched still hold the basis state's values (all bits of a complex register; the Pauli x digits
 * of a real one), so tiles that differ there stay zero and are skipped. The result equals
 * set_basis + lsg_program_run. With pass_ms non-NULL, as lsg_program_run_timed. */
int lsg_program_run_from_basis(lsg_program p, lsg_state s, int64_t index, float* pass_ms);
/* lsg_program_run_from_basis of `count` (program, register) pairs — circuits of uneven widths and
 * batches, one precision — as ONE sequence of launches: launch k carries pass k of every program
 * that has one, each program's tiles taken by its own range of the launch's CTAs (the operator
 * interpreter; a specialized program runs interpreted here, with the same results). index[i] is
 * pair i's basis state (NULL: all 0). The launches go on register 0's stream after the earlier
 * work of every register's stream, and later work on any of the registers goes after them; the
 * call does not wait (lsg_state_sync on a register waits and reports device errors). A register
 * may appear once; a program more than once only with the same basis index. With step_ms non-NULL the call waits and step_ms gets each launch's device
 * time (as many entries as the longest program has passes). Each register's result equals its
 * lsg_program_run_from_basis alone. No counterpart in the reference, which runs one circuit per
 * call (simulator.py:229-251). */
int lsg_programs_run_ragged(int32_t count, const lsg_program* programs, const lsg_state* states, const int64_t* index,
                            float* step_ms);
/* Circuit templates. lsg_program_set_data gives program p the operator data of `ops`/`pool` — the
 * same circuit template with other parameters — without planning or allocating again: the
 * operators must plan exactly as p's did (same passes, blocks, operator codes and data layout;
 * otherwise LSG_E_STATE and p is unchanged). The copy is ordered on register s's stream, after
 * its earlier work. lsg_program_graph_run is lsg_program_run_from_basis(p, s, index, NULL) as
 * one CUDA graph launch: the first call for a (register, index) pair runs the program and
 * captures basis state + passes into a graph that later calls replay; data set since stays in
 * effect (the graph reads p's device data). Neither waits. No counterpart in the reference, which
 * parses a template again for every set of `input` parameters (qasm.py:842-870) and evolves each
 * circuit from scratch (simulator.py:229-251). */
int lsg_program_set_data(lsg_program p, lsg_state s, const lsg_op* ops, int32_t nops, const double* pool,
                         int64_t pool_entries);
int lsg_program_graph_run(lsg_program p, lsg_state s, int64_t index);
/* HBM bytes (2 x tile bytes per tile visited) and tiles of one lsg_program_run_from_basis. */
int lsg_program_basis_info(lsg_program p, int64_t* bytes_per_run, int64_t* tiles_per_run);
/* Number of fused passes, and algorithmic HBM bytes of one run (2 x register bytes per pass). */
int lsg_program_info(lsg_program p, int32_t* passes, int64_t* bytes_per_run);
/* Per pass (cap >= the program's pass count; any output may be NULL): the HBM bytes one
 * lsg_program_run_from_basis moves (2 x tile bytes per tile visited; all tiles before the first
 * such run), the floating-point
 * operations per register element its operators execute (multiply or add 1, fused multiply-add 2),
 * and its register blocks. Host-side diagnostic for rooflines; no counterpart in the reference. */
int lsg_program_pass_info(lsg_program p, int32_t cap, int64_t* bytes, double* flops_per_element, int32_t* blocks);
/* Plan and launch choices of one program (0 in a field: the default for the element type, or
 * its environment knob). tile_bits: register bits per tile (a tile at most 64 KB); low_bits:
 * register bits every tile keeps contiguous (runs of at least 16 bytes); ctas: CTAs per SM the
 * specialized passes are compiled for (1-4); max_ops: operators per pass (1-192). */
typedef struct lsg_plan_opts {
    int32_t tile_bits, low_bits, ctas, max_ops;
} lsg_plan_opts;
/* lsg_program_create with explicit plan choices (the autotuner's search space). No counterpart in
 * the reference, whose kernel choices are fixed thresholds (engines.py:20-27). */
int lsg_program_create_opts(lsg_state shape, const lsg_op* ops, int32_t nops, const double* pool,
                            int64_t pool_entries, const lsg_plan_opts* opts, lsg_program* out);
/* 1 when the program's passes run as kernels specialized for it at creation (NVRTC, LSG_JIT=1),
 * 0 when the generic pass kernel interprets its operator records, negative on error. */
int lsg_program_specialized(lsg_program p);
/* 1 when the specialization policy (LSG_JIT, LSG_JIT_MIN_BYTES) takes a program whose run moves
 * `bytes_per_run` algorithmic bytes (as lsg_program_info reports), 0 when not, negative on error.
 * Lets a caller that splits one batch into several programs of the same shape keep them
 * specialized when the whole batch would be. */
int lsg_jit_wanted(int64_t bytes_per_run);
/* Host-only diagnostic (no device is touched): the CUDA source of the specialized passes a
 * program of these operators would get (into buf, at most cap bytes with the terminating zero;
 * *len = full length, 0 when the program would be interpreted), and with `compile` != 0 its NVRTC
 * compilation for sm_103a (LSG_E_ARG with the compiler log when it fails). */
int lsg_program_source(int nbits, int precision, int64_t batch, const lsg_op* ops, int32_t nops, const double* pool,
                       int64_t pool_entries, int compile, char* buf, int64_t cap, int64_t* len);
/* Independent of the register the program was created with (either may be freed first); waits for
 * the device before releasing the program's memory. */
int lsg_program_free(lsg_program p);
/* Host-only: the number of fused passes lsg_apply would run for these operators on a register of
 * nbits bits (no device is touched; used for sizing and for algorithmic-byte accounting). */
int lsg_plan(int nbits, int precision, const lsg_op* ops, int32_t nops, int32_t* passes);
/* Wait for the register's queued work; reports a device-side timeout if one occurred. */
int lsg_state_sync(lsg_state s);
/* The register's CUDA stream (a cudaStream_t), for callers that order their own work after it. */
int lsg_state_stream(lsg_state s, void** stream);

/* ---- reductions (FP64 accumulation for both precisions) -------------------------------------
 * Probabilities of member `member`: |a|^2 for a statevector register (dm_qubits = 0), the
 * clipped real diagonal for a density register of dm_qubits qubits. out has 2^n doubles; with
 * member < 0 it gets every member's, one after another (batch x 2^n).
 * Replaces Statevector.probabilities / DensityMatrix.probabilities (engines.py:207-209, :257-260). */
int lsg_probabilities(lsg_state s, int dm_qubits, int64_t member, double* out);

/* Sampling of member `member` as _sample does it (src/lucivant_sim/simulator.py:254-284):
 * marginal over `measured` (ascending qubits, m of them), FP64 prefix sum normalised by its last
 * entry, upper-bound search of `uniforms[0..shots)`, clamped. Then readout flips: for pair j
 * (pair_pos[j] = position of the qubit in `measured`), if pair_has_err[j] the flip happens when
 * flip_uniforms[e*shots + s] < (bit ? p10 : p01), e counting pairs with errors in order.
 * bits_out is shots x npairs uint8 (row-major). near_out (may be NULL) gets, per shot, 1 when
 * its uniform lies within 1e-12 of a CDF boundary (a shot a different summation order could flip).
 * Returns the number of such shots in *near_count. */
int lsg_sample(lsg_state s, int dm_qubits, int64_t member, const int32_t* measured, int32_t m,
               const double* uniforms, int64_t shots, int32_t npairs, const int32_t* pair_pos,
               const int32_t* pair_has_err, const double* pair_p01, const double* pair_p10,
               const double* flip_uniforms, uint8_t* bits_out, uint8_t* near_out, int64_t* near_count);

/* Replaces the readout branching of simulator.py:445-486 (outcome_probabilities): member 0's
 * probabilities marginalised onto `measured` (m qubits, ascending), entries <= threshold left out,
 * then final-measurement pair j (of npairs <= 30, in the circuit's order) reads measured position
 * pair_pos[j] and reports a flipped bit with probability pair_p01[j] (true 0) or pair_p10[j]
 * (true 1). out (host, 2^npairs doubles): out[e] = probability that pair j reported bit j of e for
 * every j. The caller deposits the pair bits onto their classical bits. */
int lsg_outcome_probabilities(lsg_state s, int dm_qubits, const int32_t* measured, int32_t m, int32_t npairs,
                              const int32_t* pair_pos, const double* pair_p01, const double* pair_p10, double threshold,
                              double* out);
/* <P> for Pauli terms given by x/z masks (Y sets both; qubit q = bit q), for every member.
 * out[t * batch + b]. Statevector: sum_b conj(psi[b^x]) c(b) psi[b]; density register:
 * sum_s c(s) rho[s][s^x]. Replaces the per-term loops of expectation
 * (src/lucivant_sim/simulator.py:505-527). */
int lsg_expect_pauli(lsg_state s, int dm_qubits, const uint64_t* xmask, const uint64_t* zmask,
                     int32_t nterms, double* out);

/* Probability that qubit q reads 1 in member `member` (statevector registers). Replaces
 * Statevector.probability_of_one (engines.py:185-187). */
int lsg_prob_one(lsg_state s, int qubit, int64_t member, double* out);
/* Zero the half of member `member` where qubit q != outcome and divide by sqrt(probability) when
 * probability > 0 (engines.py:195-201). */
int lsg_collapse(lsg_state s, int qubit, int outcome, double probability, int64_t member);

/* ---- trajectories ----------------------------------------------------------------------------
 * Orrery's per-shot interpreter (_trajectory, src/lucivant_sim/simulator.py:287-317; the shot
 * loop :364-371; Statevector.apply_channel / measure / reset, engines.py:159-205) as a device
 * program over a register whose members are shots. Operations are given flattened, with if/else
 * blocks bracketed by LSG_T_IF / LSG_T_ELSE / LSG_T_ENDIF. Every member draws its uniforms from a
 * cursor in the reference's order: one per noisy gate (mixture or Kraus), one per measurement or
 * reset, one more per measurement with a readout error. */
#define LSG_T_GATE 0    /* unitary: opkind is LSG_OP_MATRIX/DIAG/PERM, data as for lsg_op */
#define LSG_T_MIXTURE 1 /* mixture channel (nq <= 2), count branches: data holds count entries (re = running
                           sum of the branch probabilities in order, im = 1 for an identity branch), then
                           count dense 2^nq matrices */
#define LSG_T_KRAUS 2   /* Kraus channel (nq <= 2): count operators, dense 2^nq x 2^nq, at data */
#define LSG_T_MEASURE 3 /* qubits[0] into clbit (-1: discarded); readout != 0: one more uniform, flip with
                           p10 (read 1 as 0) or p01 */
#define LSG_T_RESET 4   /* measure qubits[0] with one uniform, then X when the outcome is 1 */
#define LSG_T_SCALE 5   /* global phase: the factor at data */
#define LSG_T_IF 6      /* holds when the count clbits listed at data (real parts, least significant first)
                           read `value`, inverted by negate */
#define LSG_T_ELSE 7
#define LSG_T_ENDIF 8

typedef struct lsg_traj_op {
    int32_t kind, opkind, nq, count;
    int32_t qubits[4];
    int32_t clbit, readout, negate, pad;
    int64_t data;
    uint64_t value;
    double p01, p10;
} lsg_traj_op;

typedef struct lsg_traj_s* lsg_traj;
int lsg_traj_create(lsg_state shape, const lsg_traj_op* ops, int32_t nops, const double* pool,
                    int64_t pool_entries, int32_t num_clbits, lsg_traj* out);
/* Upper bound of the uniforms one shot draws, and the number of compiled steps. */
int lsg_traj_info(lsg_traj t, int64_t* max_draws, int32_t* steps);
/* Serial: `shots` shots one after another on a one-member register, all drawing from one stream
 * uniforms[0..nuniforms) (at least shots x max_draws) in order, exactly as Orrery's shot loop does.
 * clbits_out: shots x ceil(num_clbits/64) words; consumed: uniforms actually drawn; near_count:
 * decisions whose uniform fell within 1e-12 of a threshold computed on the device. */
int lsg_traj_run_serial(lsg_traj t, lsg_state s, int64_t shots, const double* uniforms, int64_t nuniforms,
                        uint64_t* clbits_out, int64_t* consumed, int64_t* near_count);
/* Batched: every member is one shot drawing from its own row uniforms[b * ustride ..] (ustride >=
 * max_draws). clbits_out: batch x words; consumed: per member. */
int lsg_traj_run_batched(lsg_traj t, lsg_state s, const double* uniforms, int64_t ustride, uint64_t* clbits_out,
                         int64_t* consumed, int64_t* near_count);
int lsg_traj_free(lsg_traj t);

/* ---- stabilizer ------------------------------------------------------------------------------
 * The Aaronson-Gottesman tableau of src/lucivant_sim/stabilizer.py on the device. Gates are given
 * as codes: 0 id, 1 h, 2 s, 3 sdg, 4 x, 5 y, 6 z, 7 cx, 8 cz (the update rules of
 * stabilizer.py:224-254), or 16 + t for conjugation table t (:256-264). A table record is 65
 * bytes: the width k (1..3), then 64 entries indexed by the Pauli bits (x0 z0 x1 z1 ...), first
 * qubit most significant, each (sign << 7) | image bits in the same order. */
typedef struct lsg_cgate {
    int16_t code;  /* gate code */
    int16_t noise; /* Pauli-noise table after the gate, -1 for none (frames only) */
    int16_t a, b, c;
    int16_t nq; /* qubits of a table gate */
    int32_t pad;
} lsg_cgate;

/* Pauli noise as branches (stabilizer.py:173-187): cumulative = np.cumsum(p) / sum(p), and per
 * branch the (x, z) bits of each qubit, first qubit in the highest pair. */
typedef struct lsg_noise_table {
    int32_t k, nbranch;
    double cumulative[16];
    uint8_t label[16];
} lsg_noise_table;

typedef struct lsg_tab_s* lsg_tab;
/* |0...0> on n <= 2048 qubits (Tableau.__init__, stabilizer.py:196-208). */
int lsg_tab_create(int n, lsg_tab* out);
int lsg_tab_free(lsg_tab t);
/* Apply gates in order (noise fields ignored). */
int lsg_tab_apply(lsg_tab t, const lsg_cgate* gates, int64_t ngates, const uint8_t* tables, int32_t ntables);
/* The tableau as Orrery holds it: x, z as (n, 2n) uint8, r as (2n). */
int lsg_tab_download(lsg_tab t, uint8_t* x, uint8_t* z, uint8_t* r);
/* Tableau.support (stabilizer.py:333-365): x0 (m bytes) and the basis (rank x m bytes, may be
 * NULL) of the outcomes on `qubits`. */
int lsg_tab_support(lsg_tab t, const int32_t* qubits, int32_t m, uint8_t* x0, uint8_t* basis, int32_t* rank);
/* Gate records of a circuit held as arrays (host only, no device): gate i is of kind kind[i] (one
 * distinct gate each; kind_code / kind_nq / kind_noise per kind, as the encoder gives them for
 * that kind's gates) on qubits[3i .. 3i + arity[i]) (arity 1..3; the other slots are written 0).
 * The per-gate loop of the encoder behind Tableau gates and _frames (stabilizer.py:224-264,
 * :514-594) for the columnar form of a wide circuit. */
int lsg_cgates_from_kinds(int64_t n, const int64_t* kind, int32_t nkinds, const int16_t* kind_code,
                          const int16_t* kind_nq, const int16_t* kind_noise, const int64_t* qubits, const int64_t* arity,
                          lsg_cgate* out);
/* _frames (stabilizer.py:514-563) plus _count's readout flips (:622-643): the noisy static
 * circuit's Pauli frames over `shots`, drawing from the PCG64 generator state `rng_state`
 * (state hi, state lo, inc hi, inc lo; no uint32 buffered) in Orrery's order: the frame bits, one
 * uniform per shot per noisy gate, one per shot per readout pair with an error (pair_err >= 0).
 * bits_out: shots x nclbits outcome bytes; raw_used: 64-bit draws consumed. */
int lsg_frames_run(int n, const lsg_cgate* gates, int64_t ngates, const uint8_t* tables, int32_t ntables,
                   const lsg_noise_table* noise, int32_t nnoise, int64_t shots, const uint64_t* rng_state,
                   int32_t npairs, const int32_t* pair_qubit, const int32_t* pair_clbit, const uint8_t* pair_x0,
                   const int32_t* pair_err, const double* p01, const double* p10, int32_t nclbits,
                   uint8_t* bits_out, int64_t* raw_used);
/* _sampled (stabilizer.py:597-619) plus readout: x0 XOR basis combinations chosen by the stream's
 * uint8 integers, then the readout flips. */
int lsg_stab_sample(int m, const uint8_t* x0, const uint8_t* basis, int32_t nb, int64_t shots,
                    const uint64_t* rng_state, int32_t npairs, const int32_t* pair_pos, const int32_t* pair_clbit,
                    const int32_t* pair_err, const double* p01, const double* p10, int32_t nclbits,
                    uint8_t* bits_out, int64_t* raw_used);
/* _per_shot (stabilizer.py:653-694): dynamic Clifford circuits, one tableau per shot after the
 * noiseless prefix `prefix`, shots in order. ops: gate codes (noise = Pauli-noise table, -1 none),
 * or 100 measure (a = qubit, clbit, noise = readout row of `readout` = (p01, p10) pairs, -1 none),
 * 101 reset (a), 102 if (c = condition index, aux = op to jump to when it fails), 103 else (aux =
 * op after the matching endif), 104 endif. rng_state: 7 words (state hi/lo, inc hi/lo, the
 * buffered-uint32 flag, the buffered value, raw draws): in, the generator at the start; out, where
 * NumPy's generator would be after the same draws. clbits_out: shots x 4 words. */
typedef struct lsg_shot_op {
    int16_t code, noise, a, b, c, clbit;
    int32_t aux;
    int16_t nq, pad0;
    int32_t pad1;
} lsg_shot_op;
typedef struct lsg_shot_cond {
    int32_t n, negate;
    uint64_t value;
    int32_t bits[64];
} lsg_shot_cond;
int lsg_per_shot_run(int n, const lsg_cgate* prefix, int64_t nprefix, const lsg_shot_op* ops, int32_t nops,
                     const uint8_t* tables, int32_t ntables, const lsg_noise_table* noise, int32_t nnoise,
                     const double* readout, int32_t nreadout, const lsg_shot_cond* conds, int32_t nconds,
                     int32_t num_clbits, int64_t shots, uint64_t* rng_state, uint64_t* clbits_out);
/* Host-side check of the generator: raw draw number `index` after the state (4 words as above). */
int lsg_pcg_raw(const uint64_t* state, uint64_t index, uint64_t* out);

/* ---- allocation-free expectations ---------------------------------------------------------
 * No counterpart in the reference: an extra entry point for callers that cannot let the library
 * allocate device memory (a runtime or framework that owns the whole GPU through its own memory
 * pool and budget, or a latency-bound loop that cannot take cudaMalloc/cudaFree's device-wide
 * synchronisation). Same results as lsg_expect_pauli, but the caller passes device pointers:
 * `amplitudes` (batch members of 2^nbits complex128 or complex64 values, contiguous) and
 * `out_device` (nterms x batch doubles, out[t * batch + b]). It calls no cudaMalloc/cudaFree: its
 * only working memory is one file-scope __device__ array of LSG_NOALLOC_SCRATCH_BYTES, which every
 * GPU that loads the library holds until the process exits. The masks and nterms x batch partial
 * sums must fit in it, and one call takes at most 65,535 members; larger requests fail with
 * LSG_E_ARG, as do buffers that are not device memory of the current device. The first call on a device looks up
 * the array's device address on that device (call it once, with the device current, before any
 * latency-critical use and before any stream capture). Every call shares the array, so calls that overlap on the GPU race:
 * serialise them (one stream, or wait between calls). The call waits for its own stream before
 * returning. `stream` is a cudaStream_t (NULL: the legacy default stream). */
#define LSG_NOALLOC_SCRATCH_BYTES (1u << 20)
int lsg_expect_pauli_noalloc(const void* amplitudes, int precision, int nbits, int64_t batch, int dm_qubits,
                             const uint64_t* xmask, const uint64_t* zmask, int32_t nterms, double* out_device,
                             void* stream);

#ifdef __cplusplus
}
#endif
#endif /* LSG_H */
