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

#ifdef __cplusplus
}
#endif

#endif /* QANDLE_GB300_H */
