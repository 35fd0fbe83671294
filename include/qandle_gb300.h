/*
 * qandle_gb300.h -- C ABI of the GB300 (sm_103a) state-vector engine behind
 * qandle's front end.
 *
 * Conventions shared by every entry point:
 *   - A state is complex64 interleaved {re, im} float pairs shaped
 *     [batch][2^n], contiguous, 16-byte aligned, on the current CUDA device.
 *   - Qubit q is the reference's qubit index: it lives at bit (n-1-q) of the
 *     basis index (qandle/operators.py:549).
 *   - Gates act in the reference's row-vector convention, out = in @ M
 *     (qandle/operators.py:125-126, :289-298).
 *   - `stream` is a cudaStream_t (NULL = legacy default stream).  All work is
 *     enqueued on it; nothing synchronises unless documented.
 *   - The caller owns every buffer, including the scratch buffers whose
 *     minimum size the matching *_scratch_bytes function returns.  The
 *     library allocates no device memory on these paths.
 *   - Return value 0 = success; otherwise a QG_E* code, with a message for
 *     the calling thread in qg_last_error().
 * No entry point takes torch types; pointers are device pointers unless the
 * name says host.
 */
#ifndef QANDLE_GB300_H
#define QANDLE_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define QG_OK 0
#define QG_EINVAL 1
#define QG_ECUDA 2
#define QG_ETIMEOUT 3
#define QG_ENOMEM 4

/* Library version (major * 100 + minor). */
int qg_version(void);
/* Message of the last failed call on this host thread ("" if none). */
const char* qg_last_error(void);

/* ------------------------------------------------------------------------
 * Plain form: one HBM pass per gate, in place.
 * ------------------------------------------------------------------------ */

/* RX / RY / RZ on `qubit` by angle theta (t = theta / 2), axis 0/1/2.
 * theta_stride 0: theta[0] for all samples; 1: theta[b] per sample (the
 * reference's named / data re-uploading input).  dagger != 0 applies the
 * inverse.  Replaces BuiltRX/RY/RZ.forward, qandle/operators.py:265-298
 * (matrix builders :368-395). */
int qg_apply_rotation(void* state, int64_t batch, int n, int qubit, int axis, const float* theta,
                      int64_t theta_stride, int dagger, void* stream);

/* Fixed 2x2 complex `row_matrix` (device, 4 x {re, im}, row-major) applied as
 * state @ kron(..., row_matrix, ...).  Replaces BuiltU.forward,
 * qandle/operators.py:87-129. */
int qg_apply_matrix(void* state, int64_t batch, int n, int qubit, const void* row_matrix,
                    int dagger, void* stream);

/* Controlled 2x2: the rotation (or row matrix) on `qubit` acts only where
 * `control` is 1; the other amplitudes are kept.  Replaces
 * BuiltControlled.forward, qandle/operators.py:486-503 (the reference applies
 * the target's full matrix to the control-1 rows). */
int qg_apply_controlled_rotation(void* state, int64_t batch, int n, int control, int qubit, int axis,
                                 const float* theta, int64_t theta_stride, int dagger, void* stream);
int qg_apply_controlled_matrix(void* state, int64_t batch, int n, int control, int qubit,
                               const void* row_matrix, int dagger, void* stream);

/* Reset of `qubit` to |0> keeping the norm: for every pair of amplitudes that
 * differ in the qubit, a0 <- a0 * |(a0, a1)| / (|a0| + 1e-7), a1 <- 0.
 * Replaces BuiltReset.forward, qandle/operators.py:612-623. */
int qg_reset(void* state, int64_t batch, int n, int qubit, void* stream);

/* CNOT: out[i] = in[i ^ target] where the control bit of i is set.  Exact.
 * Replaces BuiltCNOT.forward, qandle/operators.py:536-566. */
int qg_apply_cnot(void* state, int64_t batch, int n, int control, int target, void* stream);

/* CZ: negate amplitudes with both bits set.  Exact.
 * Replaces BuiltCZ.forward, qandle/operators.py:570-598. */
int qg_apply_cz(void* state, int64_t batch, int n, int control, int target, void* stream);

/* SWAP of two qubits.  Exact.  Replaces BuiltSWAP.forward,
 * qandle/operators.py:653-677. */
int qg_apply_swap(void* state, int64_t batch, int n, int qubit_a, int qubit_b, void* stream);

/* AngleEmbedding: out = prod_j R_axis(x[b][j]) on qubits[j] applied to
 * |0..0> (the incoming state is ignored).  x row b starts at x + b *
 * x_row_stride.  qubits is a HOST array of nq entries (duplicates compose).
 * Replaces AngleEmbeddingBuilt.forward, qandle/embeddings.py:114-164. */
int64_t qg_angle_embedding_scratch_bytes(int64_t batch, int n);
int qg_angle_embedding(void* out, const float* x, int64_t x_row_stride, int64_t batch, int n,
                       const int* qubits, int nq, int axis, void* scratch, int64_t scratch_bytes,
                       void* stream);

/* AmplitudeEmbedding: out[b] = (x[b][0..len), pad_value, ..., pad_value) as
 * real amplitudes of 2^n entries, divided by max(||.||_2, 1e-12) when
 * normalize != 0 (the norm summed in fp64 in a fixed order).  Row b of x
 * starts at x + b * x_row_stride.  Replaces AmplitudeEmbeddingBuilt.forward,
 * qandle/embeddings.py:50-62 (pad then torch.nn.functional.normalize). */
int64_t qg_amplitude_embedding_scratch_bytes(int64_t batch, int64_t len);
int qg_amplitude_embedding(void* out, const float* x, int64_t x_row_stride, int64_t batch, int n, int64_t len,
                           float pad_value, int normalize, void* scratch, int64_t scratch_bytes, void* stream);

/* |psi|^2 of `count` amplitudes into float out[count].
 * Replaces MeasureAllAbsolute.forward, qandle/measurements.py:73-82. */
int qg_probs(const void* state, float* out, int64_t count, void* stream);

/* Backward of qg_probs: grad_state = 2 * grad_probs * state (torch's complex
 * gradient convention, 2 dL/dpsi*). */
int qg_probs_backward(const void* state, const float* grad_probs, void* grad_state, int64_t count,
                      void* stream);

/* P(qubit q = 0) into float out[batch][n]; sums accumulated in float64 in a
 * fixed order.  Replaces MeasureProbabilityBuilt.forward,
 * qandle/measurements.py:101-123. */
int64_t qg_measure_p0_scratch_bytes(int64_t batch, int n);
int qg_measure_p0(const void* state, float* out, int64_t batch, int n, void* scratch,
                  int64_t scratch_bytes, void* stream);

/* P0 as qg_measure_p0, for callers that cannot allocate device memory when
 * they measure (inside CUDA graphs that must not grow allocation nodes,
 * real-time loops without cudaMalloc stalls, hosts whose allocator owns all
 * device memory).  No counterpart in the reference.  The partial sums live
 * in one static device array of QG_P0_NOALLOC_MAX_PARTIALS floats (4 MiB) per
 * device, held until exit; calls needing more
 * (batch * (2^n / 2^min(n,12)) * (min(n,12) + 1)) return QG_ENOMEM.  The
 * first call on a device looks up the array's address (make it before any
 * stream capture); all calls share the array, so calls that overlap on the
 * GPU race.  The looked-up address is cached per device ordinal for the life
 * of the process: after cudaDeviceReset on a device, the cached address
 * belongs to a context that no longer exists, so do not call this entry point
 * on that device again in the same process. */
#define QG_P0_NOALLOC_MAX_PARTIALS (1 << 20)
int qg_measure_p0_noalloc(const void* state, float* out, int64_t batch, int n, void* stream);

/* Backward of qg_measure_p0: grad_state[b][i] = 2 * sum_q grad_p0[b][q] *
 * [bit (n-1-q) of i clear] * state[b][i]. */
int qg_measure_p0_backward(const void* state, const float* grad_p0, void* grad_state, int64_t batch,
                           int n, void* stream);

/* Backward of one rotation for the per-layer autograd path: dtheta =
 * 0.5 * Im <grad_out| P |out_state> per sample (per_sample = 1, dtheta[b]) or
 * summed (per_sample = 0, dtheta[0]).  grad_out is torch's complex gradient.
 * The torch autograd of BuiltParametrizedOperator.forward
 * (qandle/operators.py:289-298) computes the same quantity. */
int64_t qg_rotation_grad_scratch_bytes(int64_t batch, int n);
int qg_rotation_grad(const void* out_state, const void* grad_out, float* dtheta, int64_t batch,
                     int n, int qubit, int axis, int per_sample, void* scratch,
                     int64_t scratch_bytes, void* stream);
/* The same for a controlled rotation: only amplitudes with the control bit
 * set contribute (same scratch size). */
int qg_controlled_rotation_grad(const void* out_state, const void* grad_out, float* dtheta, int64_t batch,
                                int n, int control, int qubit, int axis, int per_sample, void* scratch,
                                int64_t scratch_bytes, void* stream);

/* ------------------------------------------------------------------------
 * Fused form: a circuit lowered once to a gate program, planned into passes
 * that each apply many gates to a shared-memory tile of 2^13 amplitudes in
 * one HBM round trip; adjoint backward over the same program.
 * Replaces the per-layer loop UnsplittedCircuit.forward
 * (qandle/qcircuit.py:163-174) and torch autograd through it.
 * ------------------------------------------------------------------------ */

/* Gate kinds (records shared with the host lowering). */
#define QG_GATE_RX 0
#define QG_GATE_RY 1
#define QG_GATE_RZ 2
#define QG_GATE_U 3
#define QG_GATE_CNOT 4
#define QG_GATE_CZ 5
#define QG_GATE_SWAP 6
#define QG_GATE_EMBED 7

/* One lowered gate.
 *   RX/RY/RZ: q0 = qubit; src 0: angle params[idx] (one for all samples),
 *             src 1: angle named[b][idx] (per sample).  t = angle / 2.
 *   U:        q0 = qubit; idx = index into the row-form 2x2 table umats;
 *             aux bit 0 set = the matrix is diagonal.
 *   CNOT/CZ:  q0 = control, q1 = target.  SWAP: q0, q1.
 *   EMBED:    AngleEmbedding; q0 = axis (0 rx, 1 ry, 2 rz), q1 = number of
 *             angles k, idx = named column of the first angle (columns
 *             idx..idx+k-1), aux = offset of its qubits in `qlist`.
 *             Gates before the last embedding are dead (it overwrites the
 *             state, qandle/embeddings.py:148-154). */
typedef struct qg_gate {
    int32_t kind, q0, q1, src, idx, aux;
} qg_gate;

#define QG_MEASURE_NONE 0  /* state out */
#define QG_MEASURE_STATE 1 /* state out (MeasureState) */
#define QG_MEASURE_PROBS 2 /* |psi|^2 [B][2^n] (MeasureAllAbsolute) */
#define QG_MEASURE_P0 3    /* P(q = 0) [B][n] (MeasureProbability) */
#define QG_MEASURE_Z 4     /* <Z_q> = P0 - P1 [B][n] */

typedef struct qg_plan_options {
    int32_t tile_bits;  /* qubits per forward tile (11..13; backward uses one less) */
    int32_t low_bits;   /* contiguous low qubits in every tile (>= 4) */
    int32_t max_high;   /* k: at most this many strided qubits per pass (0 = no limit) */
    int32_t measure;    /* QG_MEASURE_* */
    int32_t keep_state; /* also write the final state when measuring (for backward) */
    int32_t segments;   /* checkpoint segments: the forward stores the state at the
                           end of each segment but the last; the backward restarts
                           each segment from it */
    int32_t reg_bits;   /* amplitudes per thread = 2^reg_bits (4 or 5): 4 halves the
                           registers per thread and doubles the warps per tile */
    int32_t reg_search; /* qubit-remap schedule of the forward passes: 0 = greedy (each
                           new register set is the one the next gates ask for), 1 = try
                           every register set of the tile's qubits and keep the one that
                           places the most gates (backward passes always search) */
    int32_t bwd_max_grad; /* gradient-carrying rotations per backward pass (at most 64, what
                             the pass kernel's shared memory holds): 0 = the default, 28;
                             longer passes leave the instruction cache, shorter ones add
                             HBM round trips */
    int32_t fwd_max_mats; /* 2x2 slots per forward pass (a run of single-qubit gates on one
                             qubit is one slot): 0 = the default, 24 (the compiled passes
                             unroll every op, and longer ones leave the instruction cache);
                             a large value plans passes as long as the tile allows */
} qg_plan_options;

typedef struct qg_program qg_program;

typedef struct qg_program_info_t {
    int32_t num_qubits, gates, forward_passes, backward_passes, forward_ops, backward_ops;
    int32_t nparams, ncols, numats, grad_slots;
    int32_t forward_shared_slots, forward_sample_slots, backward_shared_slots, backward_sample_slots;
    int32_t segments, has_embedding;
    int64_t table_bytes;
    char summary[256];
} qg_program_info_t;

typedef struct qg_pass_info_t {
    int32_t tile_bits, nq_tile, run_bits, nfixed;
    int32_t gbit[16], fixed_gbit[32];
    int32_t op_count, init, epi, init_map[3], ckpt, psi_from_ckpt, grad_base, ngrad;
    const int32_t* ops; /* host pointer to op_count x 4 int32, valid while the program lives */
} qg_pass_info_t;

void qg_plan_options_default(qg_plan_options* opt);
/* Plan a program (host only, no GPU work).  qlist: HOST array of embedded
 * qubits.  5 <= n <= 30. */
int qg_program_create(const qg_gate* gates, int ngates, const int32_t* qlist, int n,
                      const qg_plan_options* opt, qg_program** out);
void qg_program_destroy(qg_program* prog);
int qg_program_info(const qg_program* prog, qg_program_info_t* info);
/* Inspect one planned pass (backward = 0/1). */
int qg_program_pass(const qg_program* prog, int backward, int index, qg_pass_info_t* out);
/* Matrix slots of the forward (backward = 0) or backward plan as int32
 * records {per_sample, table_index, chain_len, chain_len x {kind, src, idx,
 * dagger}}; returns the record length (copies only if cap is large enough). */
int qg_program_slots(const qg_program* prog, int backward, int32_t* out, int64_t cap);
/* Gradient slots of the backward plan as {src, idx} pairs (src 0: params,
 * 1: named column); returns the slot count. */
int qg_program_grad_targets(const qg_program* prog, int32_t* out, int64_t cap);
/* Serialise the device tables into a HOST buffer of info.table_bytes; the
 * caller copies them to device memory once and passes that pointer below. */
int qg_program_table(const qg_program* prog, void* host_out, int64_t bytes);

/* Compile the passes of `prog` for the current device: each pass's op list is
 * unrolled into its own kernel (NVRTC, sm_103a).  Afterwards
 * qg_program_forward / qg_program_forward_timed (and qg_program_backward,
 * with QG_COMPILE_BACKWARD) on this device launch the compiled kernels
 * instead of the op interpreter; results agree with the interpreter within
 * float rounding.  Identical passes compile once per
 * process.  Returns QG_ECUDA with the compiler log in qg_last_error() when
 * NVRTC is missing or fails; the interpreter then stays in use.  No
 * counterpart in the reference, whose layers run one dense matmul each
 * (qandle/qcircuit.py:163-174). */
int qg_program_compile(qg_program* prog, int flags);
/* flags: QG_COMPILE_NO_LOAD compiles every pass and discards the result (no
 * device needed: a host-side check that the program's kernels build);
 * QG_COMPILE_BACKWARD also compiles the backward passes, which
 * qg_program_backward then launches; QG_COMPILE_BACKGROUND compiles on a
 * quarter of the host's cores at a lower scheduling priority (a compile
 * beside latency-sensitive work, e.g. a serving loop).  Any host thread may
 * call it: the device's primary context is made current on it. */
#define QG_COMPILE_NO_LOAD 1
#define QG_COMPILE_BACKWARD 2
#define QG_COMPILE_BACKGROUND 4
/* 0: nothing compiled for `prog` on the current device; 1: forward passes;
 * 3: forward and backward passes. */
int qg_program_compiled(const qg_program* prog);
/* The CUDA source of compiled forward (backward = 0) or backward pass `pass`
 * (NUL-terminated) into host_out; returns the bytes needed including the
 * NUL, or -1. */
int64_t qg_program_pass_source(const qg_program* prog, int backward, int pass, char* host_out, int64_t bytes);

/* Workspace bytes for a forward (backward = 0) or backward run at `batch`. */
int64_t qg_program_workspace_bytes(const qg_program* prog, int64_t batch, int backward);

/* Forward.  state: [B][2^n]; input unless the program starts with an
 * embedding (zero_init != 0 starts from |0..0> instead), and output when the
 * plan stores the state.  params [nparams], named [B][ncols], umats
 * [numats][4] complex.  out: probs [B][2^n] or P0/<Z> [B][n] per `measure`.
 * ckpt: [segments-1][B][2^n] or NULL when segments == 1. */
int qg_program_forward(const qg_program* prog, const void* dev_table, void* workspace,
                       int64_t workspace_bytes, void* state, int64_t batch, int zero_init,
                       const float* params, const float* named, const void* umats, float* out,
                       void* ckpt, void* stream);

/* Same as qg_program_forward, and records pass_events[2p] / [2p+1]
 * (cudaEvent_t, created by the caller) on `stream` around forward pass p, so
 * a caller can time the pass kernels on the stream they run on. */
int qg_program_forward_timed(const qg_program* prog, const void* dev_table, void* workspace,
                             int64_t workspace_bytes, void* state, int64_t batch, int zero_init,
                             const float* params, const float* named, const void* umats, float* out,
                             void* ckpt, void* const* pass_events, void* stream);

/* ---- building blocks of a forward, for callers that interleave programs
 * (continuous batching): prepare (matrix tables, embedding factors), one
 * launch per pass for up to QG_MAX_JOBS independent (program, state) jobs,
 * finish (measurement reduction). ---- */
#define QG_MAX_JOBS 32

typedef struct qg_job {
    const qg_program* prog;
    const void* table;        /* device tables of prog */
    void* workspace;          /* forward workspace of this job (prepared) */
    int64_t workspace_bytes;
    void* state;              /* [batch][2^n] */
    int64_t batch;
    int32_t pass;             /* forward pass index to run */
    int32_t zero_init;        /* pass 0 starts from |0..0> */
    float* out;               /* measurement output (probs written by the last pass) */
} qg_job;

int qg_program_prepare(const qg_program* prog, const void* dev_table, void* workspace,
                       int64_t workspace_bytes, int64_t batch, const float* params, const float* named,
                       const void* umats, void* stream);
/* One kernel launch running pass jobs[i].pass of every job.  The jobs must be
 * independent (distinct states) and planned with the same tile_bits. */
int qg_jobs_run_pass(const qg_job* jobs, int njobs, void* stream);
/* Pass job->pass of one job as its own launch of the program's compiled pass
 * kernel (qg_program_compile) for the current device: the kernel
 * qg_program_forward runs for that pass.  Returns QG_EINVAL, launching
 * nothing, when that kernel is not compiled and loaded on this device.  (No
 * counterpart in the reference, which has no serving loop.) */
int qg_job_run_pass_compiled(const qg_job* job, void* stream);

int qg_program_finish(const qg_program* prog, const void* dev_table, void* workspace,
                      int64_t workspace_bytes, int64_t batch, float* out, void* stream);

/* Status word of a program workspace after the work queued on `stream`: QG_OK,
 * or QG_ETIMEOUT when a pass kernel's bounded wait on a producer / compute
 * hand-off ran out (its results are then invalid; qg_last_error() names the
 * wait that gave up, its block and tile: the workspace's first 16 bytes hold
 * status, site, block, tile).  Synchronises the stream.
 * (No reference counterpart: the reference runs no asynchronous kernels.) */
int qg_workspace_status(const void* workspace, void* stream);

/* Self-test of the bounded waits: one CTA waits on an mbarrier that nothing
 * completes, with a limit of limit_ns (at most 2e9).  Returns QG_ETIMEOUT when
 * the wait ran out and reported it (the expected outcome); the context stays
 * usable.  (No reference counterpart.) */
int qg_selftest_wait_timeout(int64_t limit_ns, void* stream);

/* FP32 roof probe for the roofline of the fused passes (no reference
 * counterpart): qg_fp32_probe_blocks() blocks of 256 threads each run
 * independent chains of packed FP32 FMAs for `iters` iterations and write one
 * float per block into out (at least qg_fp32_probe_blocks() floats).
 * *fma_count receives the FMAs the launch performs; time it with events on
 * `stream`.  Changes no device setting. */
int64_t qg_fp32_probe_blocks(void);
int qg_fp32_probe(float* out, int64_t out_floats, int64_t iters, int64_t* fma_count, void* stream);

/* Adjoint backward.  state: the forward's final state (overwritten: it is
 * un-computed gate by gate); lam: [B][2^n] buffer.  grad_out is the upstream
 * gradient of the forward output (float [B][n] for P0/<Z>, float [B][2^n]
 * for probs, complex [B][2^n] torch gradient for a state output).
 * dparams [nparams] and dnamed [B][ncols] are overwritten; dstate (optional)
 * receives torch's gradient of the input state. */
int qg_program_backward(const qg_program* prog, const void* dev_table, void* workspace,
                        int64_t workspace_bytes, void* state, void* lam, int64_t batch,
                        const float* params, const float* named, const void* umats,
                        const void* grad_out, float* dparams, float* dnamed, void* dstate,
                        const void* ckpt, void* stream);

/* Same as qg_program_backward, and records pass_events[2p] / [2p+1]
 * (cudaEvent_t, created by the caller) on `stream` around backward pass p,
 * so a caller can time the backward pass kernels on the stream they run on.
 * (No reference counterpart: the reference's backward is torch autograd
 * through dense matmuls, qandle/operators.py:230,271.) */
int qg_program_backward_timed(const qg_program* prog, const void* dev_table, void* workspace,
                              int64_t workspace_bytes, void* state, void* lam, int64_t batch,
                              const float* params, const float* named, const void* umats,
                              const void* grad_out, float* dparams, float* dnamed, void* dstate,
                              const void* ckpt, void* const* pass_events, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* QANDLE_GB300_H */
