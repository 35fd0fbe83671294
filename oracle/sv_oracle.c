/*
 * sv_oracle.c -- complex128 CPU restatement of qandle's state-vector hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the CUDA engine in
 * qandle_gb300/csrc.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg may load it.  The product path never calls it.
 *
 * It restates, gate by gate, what the reference computes with dense
 * 2^n x 2^n matrices, using O(2^n) index arithmetic instead:
 *
 *   qubit q lives at bit (n-1-q) of the basis index
 *       (qandle/operators.py:549, :582, :664; measurements.py:113-118)
 *   every gate acts as  state @ M  (row-vector convention)
 *       (qandle/operators.py:125-126, :289-298)
 *   RX/RY/RZ  M = _a * a_op(t) + _b * b_op(t),  t = theta / 2, with the
 *       buffers stored transposed  (qandle/operators.py:236-238, :265-275,
 *       :368-395)
 *   U         M = kron(..., matrix, ...)   (qandle/operators.py:101-104)
 *   CNOT      out[i] = in[i ^ (1<<t2)] when bit c2 of i is set
 *       (qandle/operators.py:546-555)
 *   CZ        out[i] = -in[i] when bits c2 and t2 are both set
 *       (qandle/operators.py:580-588)
 *   SWAP      out[i] = in[i with bits a2, b2 exchanged]
 *       (qandle/operators.py:661-671)
 *   AngleEmbedding  prod_q R_q(x_q) |0...0>, the incoming state ignored
 *       (qandle/embeddings.py:139-164)
 *   MeasureProbability  P(qubit q = 0)  (qandle/measurements.py:113-123)
 *   MeasureAllAbsolute  |psi|^2         (qandle/measurements.py:78-79)
 *
 * The gradient routine is the textbook adjoint method (reverse sweep that
 * un-computes psi and the cotangent lambda gate by gate); it is a checker for
 * the engine's adjoint kernels and is itself pinned against finite
 * differences, the parameter-shift rule and qandle's torch autograd.
 *
 * Amplitudes are interleaved doubles: st[(b * 2^n + i) * 2 + {0: re, 1: im}].
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* gate record: 6 int32 per gate {kind, q0, q1, src, idx, aux} */
enum {
    OR_RX = 0,
    OR_RY = 1,
    OR_RZ = 2,
    OR_U = 3,
    OR_CNOT = 4,
    OR_CZ = 5,
    OR_SWAP = 6,
    OR_EMBED = 7,
    OR_CROT = 8,  /* controlled rotation: q0 control, q1 target, aux axis, src/idx angle */
    OR_CU = 9,    /* controlled 2x2: q0 control, q1 target, idx matrix */
    OR_RESET = 10 /* reset of q0 */
};
/* measurement kinds for the cotangent seed */
enum { OR_SEED_P0 = 0, OR_SEED_PROBS = 1, OR_SEED_STATE = 2 };

typedef struct {
    double re, im;
} cd;

static inline cd cmul(cd a, cd b) {
    cd r = {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
    return r;
}
static inline cd cadd(cd a, cd b) {
    cd r = {a.re + b.re, a.im + b.im};
    return r;
}
static inline cd cconj(cd a) {
    cd r = {a.re, -a.im};
    return r;
}

/* Row-vector 2x2 of a rotation: the matrix M with out = in @ M on the pair
 * (in0, in1).  Follows operators.py:368-395 with the transposed storage of
 * :236-238:  RX: [[c, -is], [-is, c]];  RY: [[c, s], [-s, c]];
 * RZ: diag(e^{-it}, e^{it}). */
static void rot_row_matrix(int kind, double t, cd m[4]) {
    double c = cos(t), s = sin(t);
    memset(m, 0, 4 * sizeof(cd));
    if (kind == OR_RX) {
        m[0].re = c;
        m[1].im = -s;
        m[2].im = -s;
        m[3].re = c;
    } else if (kind == OR_RY) {
        m[0].re = c;
        m[1].re = s;
        m[2].re = -s;
        m[3].re = c;
    } else {
        m[0].re = c;
        m[0].im = -s;
        m[3].re = c;
        m[3].im = s;
    }
}

/* out = in @ m on every pair of bit position p */
static void apply_row2(cd* s, int n, int p, const cd m[4]) {
    int64_t dim = (int64_t)1 << n, st = (int64_t)1 << p;
    for (int64_t i = 0; i < dim; ++i) {
        if (i & st) continue;
        cd a0 = s[i], a1 = s[i | st];
        s[i] = cadd(cmul(a0, m[0]), cmul(a1, m[2]));
        s[i | st] = cadd(cmul(a0, m[1]), cmul(a1, m[3]));
    }
}

/* out = in @ m on the pairs of bit p whose bit cmask is set
 * (BuiltControlled.forward, qandle/operators.py:486-503). */
static void apply_row2_ctrl(cd* s, int n, int p, int64_t cmask, const cd m[4]) {
    int64_t dim = (int64_t)1 << n, st = (int64_t)1 << p;
    for (int64_t i = 0; i < dim; ++i) {
        if ((i & st) || !(i & cmask)) continue;
        cd a0 = s[i], a1 = s[i | st];
        s[i] = cadd(cmul(a0, m[0]), cmul(a1, m[2]));
        s[i | st] = cadd(cmul(a0, m[1]), cmul(a1, m[3]));
    }
}

/* Reset of bit p (BuiltReset.forward, qandle/operators.py:612-623): per pair
 * the |0> amplitude takes the pair's norm, a0 * |pair| / (|a0| + 1e-7). */
static void apply_reset(cd* s, int n, int p) {
    int64_t dim = (int64_t)1 << n, st = (int64_t)1 << p;
    for (int64_t i = 0; i < dim; ++i) {
        if (i & st) continue;
        cd a0 = s[i], a1 = s[i | st];
        double nrm = sqrt(a0.re * a0.re + a0.im * a0.im + a1.re * a1.re + a1.im * a1.im);
        double n0 = sqrt(a0.re * a0.re + a0.im * a0.im);
        double sc = nrm / (n0 + 1e-7);
        s[i].re = a0.re * sc;
        s[i].im = a0.im * sc;
        s[i | st].re = 0.0;
        s[i | st].im = 0.0;
    }
}

/* Pauli P of a rotation applied (column convention) to the pair: used for the
 * generator dU/dtheta = -i/2 P U. */
static void apply_pauli(cd* s, int n, int p, int kind) {
    int64_t dim = (int64_t)1 << n, st = (int64_t)1 << p;
    for (int64_t i = 0; i < dim; ++i) {
        if (i & st) continue;
        cd a0 = s[i], a1 = s[i | st];
        if (kind == OR_RX) {
            s[i] = a1;
            s[i | st] = a0;
        } else if (kind == OR_RY) { /* Y = [[0,-i],[i,0]] */
            cd b0 = {a1.im, -a1.re}; /* -i * a1 */
            cd b1 = {-a0.im, a0.re}; /*  i * a0 */
            s[i] = b0;
            s[i | st] = b1;
        } else { /* Z */
            s[i | st].re = -a1.re;
            s[i | st].im = -a1.im;
        }
    }
}

static double gate_angle(const int32_t* g, const double* theta, const double* named_row) {
    return g[3] == 0 ? theta[g[4]] : named_row[g[4]];
}

/* Factor of one embedded qubit: R(x)|0> as a column 2-vector
 * (first column of the column-form rotation; embeddings.py:150-154). */
static void embed_factor(int rot, double x, cd f[2]) {
    double t = x * 0.5, c = cos(t), s = sin(t);
    f[0].re = f[0].im = f[1].re = f[1].im = 0.0;
    if (rot == 0) {
        f[0].re = c;
        f[1].im = -s;
    } else if (rot == 1) {
        f[0].re = c;
        f[1].re = s;
    } else {
        f[0].re = c;
        f[0].im = -s;
    }
}

static void apply_embed(cd* s, int n, const int32_t* g, const double* named_row,
                        const int32_t* qlist) {
    int rot = g[1], k = g[2], col = g[4];
    const int32_t* qs = qlist + g[5];
    cd fac[64][2];
    int has[64];
    memset(has, 0, sizeof(has));
    /* identity start |0> per qubit, then apply each listed rotation in order
     * (duplicates compose, as the reference's matrix product does) */
    for (int q = 0; q < n; ++q) {
        fac[q][0].re = 1.0;
        fac[q][0].im = 0.0;
        fac[q][1].re = 0.0;
        fac[q][1].im = 0.0;
    }
    for (int j = 0; j < k; ++j) {
        int q = qs[j];
        cd f[2];
        embed_factor(rot, named_row[col + j], f);
        if (!has[q]) {
            fac[q][0] = f[0];
            fac[q][1] = f[1];
            has[q] = 1;
        } else {
            /* apply another rotation of the same axis to the current column */
            cd m[4];
            rot_row_matrix(rot, named_row[col + j] * 0.5, m);
            cd v0 = fac[q][0], v1 = fac[q][1];
            /* column form = transpose of the row form */
            fac[q][0] = cadd(cmul(m[0], v0), cmul(m[2], v1));
            fac[q][1] = cadd(cmul(m[1], v0), cmul(m[3], v1));
        }
    }
    int64_t dim = (int64_t)1 << n;
    for (int64_t i = 0; i < dim; ++i) {
        cd a = {1.0, 0.0};
        for (int q = 0; q < n; ++q) a = cmul(a, fac[q][(i >> (n - 1 - q)) & 1]);
        s[i] = a;
    }
}

static void apply_gate(cd* s, int n, const int32_t* g, const double* theta,
                       const double* named_row, const double* umats, const int32_t* qlist) {
    int kind = g[0];
    if (kind <= OR_RZ) {
        cd m[4];
        rot_row_matrix(kind, 0.5 * gate_angle(g, theta, named_row), m);
        apply_row2(s, n, n - 1 - g[1], m);
    } else if (kind == OR_U) {
        const double* u = umats + 8 * (int64_t)g[4];
        cd m[4] = {{u[0], u[1]}, {u[2], u[3]}, {u[4], u[5]}, {u[6], u[7]}};
        apply_row2(s, n, n - 1 - g[1], m);
    } else if (kind == OR_CNOT) {
        int64_t dim = (int64_t)1 << n;
        int64_t cm = (int64_t)1 << (n - 1 - g[1]), tm = (int64_t)1 << (n - 1 - g[2]);
        for (int64_t i = 0; i < dim; ++i)
            if ((i & cm) && !(i & tm)) {
                cd tmp = s[i];
                s[i] = s[i | tm];
                s[i | tm] = tmp;
            }
    } else if (kind == OR_CZ) {
        int64_t dim = (int64_t)1 << n;
        int64_t m = ((int64_t)1 << (n - 1 - g[1])) | ((int64_t)1 << (n - 1 - g[2]));
        for (int64_t i = 0; i < dim; ++i)
            if ((i & m) == m) {
                s[i].re = -s[i].re;
                s[i].im = -s[i].im;
            }
    } else if (kind == OR_SWAP) {
        int64_t dim = (int64_t)1 << n;
        int64_t am = (int64_t)1 << (n - 1 - g[1]), bm = (int64_t)1 << (n - 1 - g[2]);
        for (int64_t i = 0; i < dim; ++i)
            if ((i & am) && !(i & bm)) {
                int64_t j = (i ^ am) | bm;
                cd tmp = s[i];
                s[i] = s[j];
                s[j] = tmp;
            }
    } else if (kind == OR_EMBED) {
        apply_embed(s, n, g, named_row, qlist);
    } else if (kind == OR_CROT) {
        cd m[4];
        rot_row_matrix(g[5], 0.5 * gate_angle(g, theta, named_row), m);
        apply_row2_ctrl(s, n, n - 1 - g[2], (int64_t)1 << (n - 1 - g[1]), m);
    } else if (kind == OR_CU) {
        const double* u = umats + 8 * (int64_t)g[4];
        cd m[4] = {{u[0], u[1]}, {u[2], u[3]}, {u[4], u[5]}, {u[6], u[7]}};
        apply_row2_ctrl(s, n, n - 1 - g[2], (int64_t)1 << (n - 1 - g[1]), m);
    } else if (kind == OR_RESET) {
        apply_reset(s, n, n - 1 - g[1]);
    }
}

/* Inverse of a gate (U^dagger in column convention = conj-transpose of the
 * row-form matrix applied in row form). */
static void apply_gate_inverse(cd* s, int n, const int32_t* g, const double* theta,
                               const double* named_row, const double* umats) {
    int kind = g[0];
    if (kind <= OR_RZ) {
        cd m[4];
        rot_row_matrix(kind, -0.5 * gate_angle(g, theta, named_row), m);
        apply_row2(s, n, n - 1 - g[1], m);
    } else if (kind == OR_U) {
        const double* u = umats + 8 * (int64_t)g[4];
        /* row form M; inverse row form = M^dagger for unitary M */
        cd m[4] = {{u[0], -u[1]}, {u[4], -u[5]}, {u[2], -u[3]}, {u[6], -u[7]}};
        apply_row2(s, n, n - 1 - g[1], m);
    } else if (kind == OR_CROT) {
        cd m[4];
        rot_row_matrix(g[5], -0.5 * gate_angle(g, theta, named_row), m);
        apply_row2_ctrl(s, n, n - 1 - g[2], (int64_t)1 << (n - 1 - g[1]), m);
    } else if (kind == OR_CU) {
        const double* u = umats + 8 * (int64_t)g[4];
        cd m[4] = {{u[0], -u[1]}, {u[4], -u[5]}, {u[2], -u[3]}, {u[6], -u[7]}};
        apply_row2_ctrl(s, n, n - 1 - g[2], (int64_t)1 << (n - 1 - g[1]), m);
    } else {
        /* CNOT, CZ, SWAP are involutions */
        apply_gate(s, n, g, theta, named_row, umats, NULL);
    }
}

int or_version(void) { return 1; }

/* Run the gate list on every sample.  named: [B][ncols] (may be NULL when
 * ncols == 0).  nthreads <= 0 uses the OpenMP default. */
void or_run(double* st, int64_t B, int n, const int32_t* gates, int ngates, const double* theta,
            const double* named, int ncols, const double* umats, const int32_t* qlist,
            int nthreads) {
    int64_t dim = (int64_t)1 << n;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 1)
#endif
    for (int64_t b = 0; b < B; ++b) {
        cd* s = (cd*)(st + 2 * b * dim);
        const double* nr = ncols > 0 ? named + b * ncols : NULL;
        for (int k = 0; k < ngates; ++k) apply_gate(s, n, gates + 6 * k, theta, nr, umats, qlist);
    }
    (void)nthreads;
}

/* P(qubit q = 0) per sample: out[b][q] */
void or_measure_p0(const double* st, int64_t B, int n, double* out) {
    int64_t dim = (int64_t)1 << n;
    for (int64_t b = 0; b < B; ++b) {
        const cd* s = (const cd*)(st + 2 * b * dim);
        for (int q = 0; q < n; ++q) {
            int64_t m = (int64_t)1 << (n - 1 - q);
            double acc = 0.0;
            for (int64_t i = 0; i < dim; ++i)
                if (!(i & m)) acc += s[i].re * s[i].re + s[i].im * s[i].im;
            out[b * n + q] = acc;
        }
    }
}

void or_probs(const double* st, int64_t count, double* out) {
    for (int64_t i = 0; i < count; ++i) out[i] = st[2 * i] * st[2 * i] + st[2 * i + 1] * st[2 * i + 1];
}

/* Adjoint gradient.  psi0: [B][2^n] input state (ignored when the first gate
 * is an embedding).  seed_kind selects how the upstream gradient `gout`
 * enters:  P0 -> gout [B][n] = dL/dP0;  PROBS -> gout [B][2^n] = dL/dp;
 * STATE -> gout [B][2^n] complex = torch's grad (2 dL/dpsi*).
 * Outputs: dtheta [ntheta] (summed over samples), dnamed [B][ncols],
 * dpsi0 [B][2^n] complex (torch convention 2 dL/dpsi0*), any may be NULL.
 * dL/dangle = Im(<lambda| P |psi>) at each rotation, lambda = dL/dpsi*. */
void or_adjoint(const double* psi0, int64_t B, int n, const int32_t* gates, int ngates,
                const double* theta, int ntheta, const double* named, int ncols,
                const double* umats, const int32_t* qlist, int seed_kind, const double* gout,
                double* dtheta, double* dnamed, double* dpsi0, int nthreads) {
    int64_t dim = (int64_t)1 << n;
    double* dth_all = (double*)calloc((size_t)B * (ntheta > 0 ? ntheta : 1), sizeof(double));
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 1)
#endif
    for (int64_t b = 0; b < B; ++b) {
        cd* psi = (cd*)malloc(sizeof(cd) * dim);
        cd* lam = (cd*)malloc(sizeof(cd) * dim);
        cd* tmp = (cd*)malloc(sizeof(cd) * dim);
        const double* nr = ncols > 0 ? named + b * ncols : NULL;
        double* dnr = (dnamed && ncols > 0) ? dnamed + b * ncols : NULL;
        double* dth = dth_all + b * (ntheta > 0 ? ntheta : 1);
        if (psi0)
            memcpy(psi, psi0 + 2 * b * dim, sizeof(cd) * dim);
        else {
            memset(psi, 0, sizeof(cd) * dim);
            psi[0].re = 1.0;
        }
        for (int k = 0; k < ngates; ++k) apply_gate(psi, n, gates + 6 * k, theta, nr, umats, qlist);
        /* cotangent seed lambda = dL/dpsi* */
        if (seed_kind == OR_SEED_P0) {
            const double* g = gout + b * n;
            for (int64_t i = 0; i < dim; ++i) {
                double w = 0.0;
                for (int q = 0; q < n; ++q)
                    if (!((i >> (n - 1 - q)) & 1)) w += g[q];
                lam[i].re = w * psi[i].re;
                lam[i].im = w * psi[i].im;
            }
        } else if (seed_kind == OR_SEED_PROBS) {
            const double* g = gout + b * dim;
            for (int64_t i = 0; i < dim; ++i) {
                lam[i].re = g[i] * psi[i].re;
                lam[i].im = g[i] * psi[i].im;
            }
        } else {
            const double* g = gout + 2 * b * dim;
            for (int64_t i = 0; i < dim; ++i) {
                lam[i].re = 0.5 * g[2 * i];
                lam[i].im = 0.5 * g[2 * i + 1];
            }
        }
        for (int k = ngates - 1; k >= 0; --k) {
            const int32_t* g = gates + 6 * k;
            int kind = g[0];
            if (kind <= OR_RZ || kind == OR_CROT) {
                /* psi is the state after the gate: Im <lam| P |psi>, over the
                 * control-1 amplitudes for a controlled rotation */
                const int axis = kind == OR_CROT ? g[5] : kind;
                const int tq = kind == OR_CROT ? g[2] : g[1];
                const int64_t cm = kind == OR_CROT ? ((int64_t)1 << (n - 1 - g[1])) : 0;
                memcpy(tmp, psi, sizeof(cd) * dim);
                apply_pauli(tmp, n, n - 1 - tq, axis);
                double acc = 0.0;
                for (int64_t i = 0; i < dim; ++i)
                    if ((i & cm) == cm) acc += cmul(cconj(lam[i]), tmp[i]).im;
                if (g[3] == 0)
                    dth[g[4]] += acc;
                else if (dnr)
                    dnr[g[4]] += acc;
            }
            if (kind == OR_EMBED) {
                /* state after the embedding is a product state; each listed
                 * rotation's generator acts on it directly */
                int rot = g[1], kq = g[2], col = g[4];
                const int32_t* qs = qlist + g[5];
                for (int j = 0; j < kq; ++j) {
                    memcpy(tmp, psi, sizeof(cd) * dim);
                    apply_pauli(tmp, n, n - 1 - qs[j], rot);
                    double acc = 0.0;
                    for (int64_t i = 0; i < dim; ++i) acc += cmul(cconj(lam[i]), tmp[i]).im;
                    if (dnr) dnr[col + j] += acc;
                }
                /* the embedding discards the incoming state: nothing flows back */
                memset(lam, 0, sizeof(cd) * dim);
                break;
            }
            apply_gate_inverse(psi, n, g, theta, nr, umats);
            apply_gate_inverse(lam, n, g, theta, nr, umats);
        }
        if (dpsi0) {
            double* d = dpsi0 + 2 * b * dim;
            for (int64_t i = 0; i < dim; ++i) {
                d[2 * i] = 2.0 * lam[i].re;
                d[2 * i + 1] = 2.0 * lam[i].im;
            }
        }
        free(psi);
        free(lam);
        free(tmp);
    }
    if (dtheta && ntheta > 0) {
        for (int j = 0; j < ntheta; ++j) {
            double acc = 0.0;
            for (int64_t b = 0; b < B; ++b) acc += dth_all[b * ntheta + j];
            dtheta[j] = acc;
        }
    }
    free(dth_all);
    (void)nthreads;
}
