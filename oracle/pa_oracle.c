/*
 * pa_oracle.c -- CPU oracle for the affine-gap (Gotoh) score-only pairwise alignment.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker the GPU path is compared
 * against; it is never part of the product path.  Only tests/, the smoke()
 * check in __graft_entry__.py and bench.py's CPU-baseline / reference legs may
 * load it.  The product library (pairwise_aligner_gb300) does not link it and
 * fails loudly when its own CUDA library is missing.
 *
 * Two entry families:
 *
 *  1. pa_oracle_align / pa_oracle_align_batch -- a scalar restatement of the
 *     reference's scalar path (cfg::score_model_unitary), int64 internally,
 *     plus end coordinates under this project's tie-break convention.
 *       - recurrence: include/pairwise_aligner/affine/affine_dp_algorithm.hpp:133-156
 *       - border cells: include/pairwise_aligner/affine/affine_initialisation_strategy.hpp:38-51
 *       - local clamp of the diagonal term: include/pairwise_aligner/matrix/dp_matrix_local.hpp:39-47
 *       - substitution: include/pairwise_aligner/score_model/score_model_unitary.hpp:52-59
 *         or, with a matrix, include/pairwise_aligner/score_model/score_model_matrix.hpp:53-63
 *         (score = matrix[rank(sequence1 symbol) * dim + rank(sequence2 symbol)], the
 *         ranks from the symbol list as in configuration/score_model_matrix.hpp:203-222)
 *       - global result (+ free trailing row/column): include/pairwise_aligner/tracker/tracker_global_scalar.hpp:36-61
 *       - local result (max over all cells, lowest() when empty): include/pairwise_aligner/tracker/tracker_local_scalar.hpp:38-49
 *     Parity is pinned against the reference's hand-written golden scores
 *     (the test/unit/affine scalar tests) by tests/test_oracle_golden.py.
 *
 *  2. pa_oracle_simd_batch -- a multi-threaded inter-sequence SIMD port of the
 *     reference's SIMD paths: one alignment per vector lane, 16-byte GCC vector
 *     extensions (native on x86 SSE2 and Arm NEON), pthreads over batches.
 *     Scores only, like the reference.  It is the timed CPU baseline where the
 *     reference itself can not be built.  Lane widths:
 *       - local alignment: 16 byte lanes per vector, as the reference's
 *         saturated int8 model (cfg::score_model_unitary_simd_saturated,
 *         configuration/score_model_unitary_simd_saturated.hpp:47-191), where
 *         saturation at the low end implements the local clamp
 *         (matrix/dp_vector_saturated_local.hpp:105-115).  Here the bytes hold
 *         the true scores, floored at 0; a lane whose best score reaches the top
 *         of the byte range is redone in int16 lanes (the reference rebases
 *         instead, matrix/dp_matrix_column_saturated_local.hpp:65-84);
 *       - otherwise 8 int16 lanes (cfg::score_model_unitary_simd<int16_t>,
 *         configuration/score_model_unitary_simd.hpp:51-137), or 4 int32 lanes
 *         for pairs whose scores could overflow int16.
 *
 * End-coordinate convention (the reference computes none: every tracker has
 * "TODO: optimal_coordinate()"): 1-based (i, j) = (end in sequence1, end in
 * sequence2) of the best cell; ties go to the smallest i, then the smallest j.
 * Local: a best score of 0 reports (0, 0); an empty input reports INT32_MIN and
 * (0, 0).  Global: the candidate cells are (m, n), plus the last row (m, 0..n)
 * when the trailing row gap is free, plus the last column (0..m, n) when the
 * trailing column gap is free.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <pthread.h>

#define PA_ORACLE_OK 0
#define PA_ORACLE_EINVAL 1
#define PA_ORACLE_ENOMEM 2

typedef struct pa_oracle_cfg {
    int32_t match;              /* score of a == b                       */
    int32_t mismatch;           /* score of a != b                       */
    int32_t gap_open;           /* gap of length k scores open + k * ext */
    int32_t gap_extension;
    int32_t local;              /* 1: method_local (all end gaps free)   */
    int32_t first_column_free;  /* leading gap in sequence1 free (H(i,0) = 0) */
    int32_t first_row_free;     /* leading gap in sequence2 free (H(0,j) = 0) */
    int32_t last_column_free;   /* result may end in column n            */
    int32_t last_row_free;      /* result may end in row m               */
    int32_t dim;                /* substitution matrix: 0 = unitary scores */
    const int32_t *matrix;      /* dim x dim, row = sequence1 symbol       */
    const int16_t *rank;        /* 256 entries: symbol -> rank, -1 invalid */
} pa_oracle_cfg;

static inline int64_t substitute(const pa_oracle_cfg *c, uint8_t a, uint8_t b)
{
    if (c->dim) return c->matrix[c->rank[a] * c->dim + c->rank[b]];
    return a == b ? c->match : c->mismatch;
}

/* With a matrix every symbol must have a rank (the reference asserts it). */
static int symbols_valid(const pa_oracle_cfg *c, const uint8_t *s, uint64_t len)
{
    if (!c->dim) return 1;
    if (!c->matrix || !c->rank || c->dim < 0) return 0;
    for (uint64_t k = 0; k < len; ++k)
        if (c->rank[s[k]] < 0 || c->rank[s[k]] >= c->dim) return 0;
    return 1;
}

static inline int64_t max64(int64_t a, int64_t b) { return a > b ? a : b; }

/* Border cell k of the first row (order = row) or first column (order = column).
 * Index 0 -> (0, open+ext); k > 0 penalised -> (open + ext*k, that + open + ext);
 * free -> (0, open+ext).   affine_initialisation_strategy.hpp:38-51 */
static inline void border_cell(const pa_oracle_cfg *c, int free_rule, uint64_t k, int64_t *h, int64_t *gap)
{
    int64_t goe = (int64_t)c->gap_open + c->gap_extension;
    int64_t first = 0;
    if (!free_rule && k > 0)
        first = (int64_t)c->gap_open + (int64_t)c->gap_extension * (int64_t)k;
    *h = first;
    *gap = first + goe;
}

/* Scalar Gotoh.  Rows i run over sequence1 (the reference's "column sequence"),
 * columns j over sequence2.  vgap[j] is the vertical gap carried down column j
 * (the reference's row-cell .second); hgap is the horizontal gap carried along
 * row i (the reference's column-cell .second).  affine_dp_algorithm.hpp:149-155 */
int pa_oracle_align(const pa_oracle_cfg *c, const uint8_t *s1, uint64_t m, const uint8_t *s2, uint64_t n,
                    int64_t *score, int64_t *end1, int64_t *end2)
{
    if (!c || !score || !end1 || !end2) return PA_ORACLE_EINVAL;
    if (!symbols_valid(c, s1, m) || !symbols_valid(c, s2, n)) return PA_ORACLE_EINVAL;
    const int local = c->local != 0;
    const int first_col_free = local || c->first_column_free;
    const int first_row_free = local || c->first_row_free;
    const int last_col_free = !local && c->last_column_free;
    const int last_row_free = !local && c->last_row_free;
    const int64_t goe = (int64_t)c->gap_open + c->gap_extension;
    const int64_t ext = c->gap_extension;

    int64_t *hrow = (int64_t *)malloc(sizeof(int64_t) * (n + 1));
    int64_t *vgap = (int64_t *)malloc(sizeof(int64_t) * (n + 1));
    if (!hrow || !vgap) { free(hrow); free(vgap); return PA_ORACLE_ENOMEM; }
    for (uint64_t j = 0; j <= n; ++j) border_cell(c, first_row_free, j, &hrow[j], &vgap[j]);

    /* result bookkeeping */
    int64_t best = INT64_MIN, bi = 0, bj = 0;
    int have = 0;
    if (!local) {
        if (last_col_free) { best = hrow[n]; bi = 0; bj = n; have = 1; }  /* H(0, n) */
        if (m == 0) {                                                       /* H(0, n) is the corner */
            if (!have || hrow[n] > best) { best = hrow[n]; bi = 0; bj = n; }
            have = 1;
            if (last_row_free)                                              /* row m = 0 */
                for (uint64_t j = 0; j <= n; ++j)
                    if (hrow[j] > best || (hrow[j] == best && (0 < bi || (0 == bi && (int64_t)j < bj)))) {
                        best = hrow[j]; bi = 0; bj = (int64_t)j;
                    }
        }
    }

    for (uint64_t i = 1; i <= m; ++i) {
        int64_t hc, hgap;
        border_cell(c, first_col_free, i, &hc, &hgap);
        int64_t diag = hrow[0];
        hrow[0] = hc;
        const uint8_t a = s1[i - 1];
        for (uint64_t j = 1; j <= n; ++j) {
            int64_t d = diag + substitute(c, a, s2[j - 1]);
            if (local) d = max64(d, 0);                       /* dp_matrix_local.hpp:39-47 */
            int64_t h = max64(max64(d, vgap[j]), hgap);
            diag = hrow[j];
            hrow[j] = h;
            if (local && h > best) { best = h; bi = (int64_t)i; bj = (int64_t)j; }
            int64_t hoe = h + goe;
            vgap[j] = max64(vgap[j] + ext, hoe);
            hgap = max64(hgap + ext, hoe);
        }
        if (!local && last_col_free) {                       /* H(i, n); (i, n) beats later rows on ties */
            if (hrow[n] > best) { best = hrow[n]; bi = (int64_t)i; bj = (int64_t)n; }
        }
    }

    if (local) {
        if (m == 0 || n == 0) { *score = INT32_MIN; *end1 = 0; *end2 = 0; }   /* tracker_local_scalar.hpp:38 */
        else if (best <= 0) { *score = best; *end1 = 0; *end2 = 0; }
        else { *score = best; *end1 = bi; *end2 = bj; }
    } else {
        if (m > 0) {
            /* (m, n) and, with a free trailing row, the last row (m, 0..n). */
            if (last_row_free) {
                for (uint64_t j = 0; j <= n; ++j) {
                    int better = !have || hrow[j] > best ||
                                 (hrow[j] == best && ((int64_t)m < bi || ((int64_t)m == bi && (int64_t)j < bj)));
                    if (better) { best = hrow[j]; bi = (int64_t)m; bj = (int64_t)j; have = 1; }
                }
            } else {
                int better = !have || hrow[n] > best ||
                             (hrow[n] == best && ((int64_t)m < bi || ((int64_t)m == bi && (int64_t)n < bj)));
                if (better) { best = hrow[n]; bi = (int64_t)m; bj = (int64_t)n; have = 1; }
            }
        }
        *score = best; *end1 = bi; *end2 = bj;
    }
    free(hrow); free(vgap);
    return PA_ORACLE_OK;
}

/* Traceback (beyond the reference, whose trackers report no coordinates or path):
 * the optimal alignment as SAM-style ops over the same recurrence and end cell as
 * pa_oracle_align.  Full int64 matrices, so for small cases only.
 *
 * States: H (any), P (a gap along sequence1: op 'D', consumes a_i), Q (a gap along
 * sequence2: op 'I', consumes b_j).  P(i,j) = max(P(i-1,j) + ext, H(i-1,j) + open + ext),
 * P(1,j) = H(0,j) + open + ext; Q likewise along j (the reference's vertical / horizontal
 * gap cells, affine_dp_algorithm.hpp:149-155, borders affine_initialisation_strategy.hpp:38-51).
 * Tie-break convention:
 *   - H(i,j): local and H == 0 -> the path starts after (i,j); else the diagonal if it
 *     attains H, else P, else Q;
 *   - P / Q: the gap opens at the previous cell unless extending is strictly better;
 *   - borders: (0,j) ends the path with j 'I' ops unless the leading row gap is free
 *     (then the path begins at (0,j)); (i,0) likewise with 'D' and the leading column.
 * '=' when the aligned symbols are equal, 'X' otherwise (with a matrix too).
 * ops receives n_ops <= m + n characters in path order; begin = the 0-based cell the
 * path starts after; end = the same end cell as pa_oracle_align (0,0 and no ops when the
 * local score is <= 0 or a sequence is empty). */
int pa_oracle_traceback(const pa_oracle_cfg *c, const uint8_t *s1, uint64_t m, const uint8_t *s2, uint64_t n,
                        int64_t *score, int64_t *begin1, int64_t *begin2, int64_t *end1, int64_t *end2,
                        uint8_t *ops, int64_t *n_ops)
{
    if (!c || !score || !begin1 || !begin2 || !end1 || !end2 || !ops || !n_ops) return PA_ORACLE_EINVAL;
    int rc = pa_oracle_align(c, s1, m, s2, n, score, end1, end2);
    if (rc) return rc;
    *begin1 = *begin2 = 0;
    *n_ops = 0;
    const int local = c->local != 0;
    if (local && (m == 0 || n == 0 || *score <= 0)) return PA_ORACLE_OK;
    const int first_col_free = local || c->first_column_free;
    const int first_row_free = local || c->first_row_free;
    const int64_t goe = (int64_t)c->gap_open + c->gap_extension, ext = c->gap_extension;
    const uint64_t W = n + 1;
    int64_t *H = (int64_t *)malloc(sizeof(int64_t) * (m + 1) * W);
    int64_t *P = (int64_t *)malloc(sizeof(int64_t) * (m + 1) * W);
    int64_t *Q = (int64_t *)malloc(sizeof(int64_t) * (m + 1) * W);
    if (!H || !P || !Q) { free(H); free(P); free(Q); return PA_ORACLE_ENOMEM; }
    for (uint64_t j = 0; j <= n; ++j) { int64_t g; border_cell(c, first_row_free, j, &H[j], &g); P[j] = g; Q[j] = g; }
    for (uint64_t i = 1; i <= m; ++i) {
        int64_t g;
        border_cell(c, first_col_free, i, &H[i * W], &g);
        P[i * W] = g; Q[i * W] = g;
        for (uint64_t j = 1; j <= n; ++j) {
            /* P(i,j), Q(i,j): the gap states entering (i,j); row 0 / column 0 hold H + goe */
            const int64_t p = i == 1 ? H[j] + goe : max64(P[(i - 1) * W + j] + ext, H[(i - 1) * W + j] + goe);
            const int64_t q = j == 1 ? H[i * W] + goe : max64(Q[i * W + j - 1] + ext, H[i * W + j - 1] + goe);
            int64_t d = H[(i - 1) * W + j - 1] + substitute(c, s1[i - 1], s2[j - 1]);
            if (local) d = max64(d, 0);
            P[i * W + j] = p;
            Q[i * W + j] = q;
            H[i * W + j] = max64(max64(d, p), q);
        }
    }
    /* walk back from the end cell; ops written in reverse, then flipped */
    int64_t i = *end1, j = *end2, k = 0;
    int state = 0;                                           /* 0 H, 1 P, 2 Q */
    for (;;) {
        if (state == 0) {
            if (i == 0 || j == 0) {                          /* a border cell */
                if (i == 0 && j > 0 && !first_row_free) { while (j > 0) { ops[k++] = 'I'; --j; } }
                else if (j == 0 && i > 0 && !first_col_free) { while (i > 0) { ops[k++] = 'D'; --i; } }
                break;
            }
            const int64_t h = H[i * W + j];
            if (local && h == 0) break;
            int64_t d = H[(i - 1) * W + j - 1] + substitute(c, s1[i - 1], s2[j - 1]);
            if (local) d = max64(d, 0);
            if (h == d) { ops[k++] = s1[i - 1] == s2[j - 1] ? '=' : 'X'; --i; --j; }
            else if (h == P[i * W + j]) state = 1;
            else state = 2;
        } else if (state == 1) {                             /* P(i,j): 'D', to (i-1, j) */
            const int64_t p = P[i * W + j];
            ops[k++] = 'D';
            const int ext_better = i > 1 && P[(i - 1) * W + j] + ext > H[(i - 1) * W + j] + goe;
            (void)p;
            --i;
            state = ext_better ? 1 : 0;
        } else {                                             /* Q(i,j): 'I', to (i, j-1) */
            ops[k++] = 'I';
            const int ext_better = j > 1 && Q[i * W + j - 1] + ext > H[i * W + j - 1] + goe;
            --j;
            state = ext_better ? 2 : 0;
        }
    }
    *begin1 = i;
    *begin2 = j;
    for (int64_t a = 0, b = k - 1; a < b; ++a, --b) { uint8_t t = ops[a]; ops[a] = ops[b]; ops[b] = t; }
    *n_ops = k;
    free(H); free(P); free(Q);
    return PA_ORACLE_OK;
}

/* H(row, 0..n) of the global recurrence (the scalar DP above stopped after
 * `row` rows of sequence1); out has n + 1 entries.  Used to check the band
 * labels: the label of checkpoint row r is argmax_j H(r, j) + H'(m - r, n - j)
 * with H' the same DP on both sequences reversed. */
int pa_oracle_row(const pa_oracle_cfg *c, const uint8_t *s1, uint64_t m, const uint8_t *s2, uint64_t n,
                  uint64_t row, int64_t *out)
{
    if (!c || !out || row > m || c->local) return PA_ORACLE_EINVAL;
    if (!symbols_valid(c, s1, m) || !symbols_valid(c, s2, n)) return PA_ORACLE_EINVAL;
    const int64_t goe = (int64_t)c->gap_open + c->gap_extension, ext = c->gap_extension;
    int64_t *vgap = (int64_t *)malloc(sizeof(int64_t) * (n + 1));
    if (!vgap) return PA_ORACLE_ENOMEM;
    for (uint64_t j = 0; j <= n; ++j) border_cell(c, c->first_row_free, j, &out[j], &vgap[j]);
    for (uint64_t i = 1; i <= row; ++i) {
        int64_t hc, hgap;
        border_cell(c, c->first_column_free, i, &hc, &hgap);
        int64_t diag = out[0];
        out[0] = hc;
        for (uint64_t j = 1; j <= n; ++j) {
            int64_t h = max64(max64(diag + substitute(c, s1[i - 1], s2[j - 1]), vgap[j]), hgap);
            diag = out[j];
            out[j] = h;
            int64_t hoe = h + goe;
            vgap[j] = max64(vgap[j] + ext, hoe);
            hgap = max64(hgap + ext, hoe);
        }
    }
    free(vgap);
    return PA_ORACLE_OK;
}

/* ------------------------------------------------------------------------- */
/* batch driver over (bytes, offsets) -- the same layout the C-ABI takes       */
/* ------------------------------------------------------------------------- */

typedef struct {
    const pa_oracle_cfg *cfg;
    const uint8_t *s1; const uint64_t *off1;
    const uint8_t *s2; const uint64_t *off2;
    uint64_t begin, end, stride;
    int64_t *scores, *end1, *end2;
    int rc;
} scalar_job;

static void *scalar_worker(void *p)
{
    scalar_job *jb = (scalar_job *)p;
    for (uint64_t k = jb->begin; k < jb->end; k += jb->stride) {
        int64_t sc, e1, e2;
        int rc = pa_oracle_align(jb->cfg, jb->s1 + jb->off1[k], jb->off1[k + 1] - jb->off1[k],
                                 jb->s2 + jb->off2[k], jb->off2[k + 1] - jb->off2[k], &sc, &e1, &e2);
        if (rc) { jb->rc = rc; return NULL; }
        jb->scores[k] = sc;
        if (jb->end1) jb->end1[k] = e1;
        if (jb->end2) jb->end2[k] = e2;
    }
    return NULL;
}

int pa_oracle_align_batch(const pa_oracle_cfg *c, const uint8_t *s1, const uint64_t *off1,
                          const uint8_t *s2, const uint64_t *off2, uint64_t n_pairs,
                          int64_t *scores, int64_t *end1, int64_t *end2, int nthreads)
{
    if (!c || !scores || (n_pairs && (!off1 || !off2))) return PA_ORACLE_EINVAL;
    if (nthreads < 1) nthreads = 1;
    if ((uint64_t)nthreads > n_pairs) nthreads = n_pairs ? (int)n_pairs : 1;
    scalar_job *jobs = (scalar_job *)calloc((size_t)nthreads, sizeof(scalar_job));
    pthread_t *th = (pthread_t *)calloc((size_t)nthreads, sizeof(pthread_t));
    if (!jobs || !th) { free(jobs); free(th); return PA_ORACLE_ENOMEM; }
    for (int t = 0; t < nthreads; ++t) {
        jobs[t] = (scalar_job){c, s1, off1, s2, off2, (uint64_t)t, n_pairs, (uint64_t)nthreads,
                               scores, end1, end2, 0};
    }
    for (int t = 1; t < nthreads; ++t) pthread_create(&th[t], NULL, scalar_worker, &jobs[t]);
    scalar_worker(&jobs[0]);
    int rc = jobs[0].rc;
    for (int t = 1; t < nthreads; ++t) { pthread_join(th[t], NULL); if (jobs[t].rc) rc = jobs[t].rc; }
    free(jobs); free(th);
    return rc;
}

/* ------------------------------------------------------------------------- */
/* inter-sequence SIMD port (CPU baseline), scores only                        */
/* ------------------------------------------------------------------------- */

/* Two lane types, as the reference's fixed-width SIMD model offers them
 * (score_model_unitary_simd<int16_t|int32_t>, score_model_unitary_simd.hpp:51-137):
 * int16 lanes for pairs whose scores fit int16, int32 lanes for the rest.  The vectors are
 * 16 bytes, the width both baseline ISAs have natively (SSE2 on x86-64, NEON on AArch64):
 * GCC lowers wider generic vectors to scalar code where the target lacks them, which made an
 * earlier 32-byte build 17x slower per thread than its AVX2 build. */
typedef int16_t v8s __attribute__((vector_size(16)));
typedef int32_t v4i __attribute__((vector_size(16)));
typedef uint8_t v16u __attribute__((vector_size(16)));

typedef struct {
    const pa_oracle_cfg *cfg;
    const uint8_t *s1; const uint64_t *off1;
    const uint8_t *s2; const uint64_t *off2;
    const uint32_t *order;        /* pairs sorted by shape */
    uint64_t n_pairs;
    uint64_t next_batch;          /* shared work counter   */
    pthread_mutex_t lock;
    int32_t *scores;
    uint8_t *redo;                /* byte lanes: pairs whose best score reached the byte limit */
    int rc;
} simd_ctx;

/* One batch of up to L pairs, one pair per lane (VT: L lanes of ST).  Like the reference's
 * bulk vectors (dp_vector_bulk.hpp:83-103) the lanes are padded to the longest pair; padding
 * symbols (0x200 in sequence1, 0x300 in sequence2) never match a byte, and padded cells
 * never feed a real cell, so only the per-lane result cell needs care.  Both sequences are
 * widened to lane vectors once per batch, so the inner loop is vector operations only. */
/* lane-wise max of two vectors (C has no vector ?:; the comparison is an all-ones lane mask) */
#define PA_VMAX(VT, A, B) ({ VT a_ = (A), b_ = (B); VT m_ = (VT)(a_ > b_); (a_ & m_) | (b_ & ~m_); })

#define PA_SIMD_BATCH(FN, VT, ST, L, ST_MIN)                                                        \
static int FN(simd_ctx *x, const uint32_t *ids, int lanes, VT *qvec, VT *tvec, VT *hrow, VT *vgap,  \
              size_t cap_n)                                                                        \
{                                                                                                  \
    const pa_oracle_cfg *c = x->cfg;                                                              \
    const int local = c->local != 0;                                                              \
    uint64_t mmax = 0, nmax = 0, ml[L], nl[L];                                                    \
    for (int l = 0; l < L; ++l) {                                                                 \
        uint32_t k = ids[l < lanes ? l : 0];                                                      \
        ml[l] = x->off1[k + 1] - x->off1[k];                                                      \
        nl[l] = x->off2[k + 1] - x->off2[k];                                                      \
        if (ml[l] > mmax) mmax = ml[l];                                                           \
        if (nl[l] > nmax) nmax = nl[l];                                                           \
    }                                                                                              \
    if (nmax + 1 > cap_n || mmax + 1 > cap_n) return PA_ORACLE_ENOMEM;                            \
    for (int l = 0; l < L; ++l) {                                                                 \
        uint32_t k = ids[l < lanes ? l : 0];                                                      \
        const uint8_t *a = x->s1 + x->off1[k], *b = x->s2 + x->off2[k];                          \
        for (uint64_t i = 0; i < mmax; ++i) qvec[i][l] = (ST)(i < ml[l] ? a[i] : 0x200);         \
        for (uint64_t j = 0; j < nmax; ++j) tvec[j][l] = (ST)(j < nl[l] ? b[j] : 0x300);         \
    }                                                                                              \
    const ST goe = (ST)(c->gap_open + c->gap_extension), ext = (ST)c->gap_extension;             \
    const int fcf = local || c->first_column_free, frf = local || c->first_row_free;             \
    VT vgoe, vext, vmatch, vmis, zero, best;                                                      \
    for (int l = 0; l < L; ++l) {                                                                 \
        vgoe[l] = goe; vext[l] = ext; vmatch[l] = (ST)c->match; vmis[l] = (ST)c->mismatch;       \
        zero[l] = 0; best[l] = ST_MIN;                                                            \
    }                                                                                              \
    for (uint64_t j = 0; j <= nmax; ++j) {                                                        \
        ST h = (!frf && j > 0) ? (ST)(c->gap_open + c->gap_extension * (int64_t)j) : 0;          \
        for (int l = 0; l < L; ++l) { hrow[j][l] = h; vgap[j][l] = (ST)(h + goe); }              \
    }                                                                                              \
    int32_t res[L];                                                                                \
    for (int l = 0; l < L; ++l) if (!local && ml[l] == 0) res[l] = hrow[nl[l]][l];               \
    for (uint64_t i = 1; i <= mmax; ++i) {                                                        \
        ST hc = (!fcf) ? (ST)(c->gap_open + c->gap_extension * (int64_t)i) : 0;                  \
        VT hgap, diag = hrow[0];                                                                  \
        for (int l = 0; l < L; ++l) { hgap[l] = (ST)(hc + goe); hrow[0][l] = hc; }               \
        const VT qa = qvec[i - 1];                                                                \
        for (uint64_t j = 1; j <= nmax; ++j) {                                                    \
            VT eq = (VT)(qa == tvec[j - 1]);                                                      \
            VT d = diag + ((vmatch & eq) | (vmis & ~eq));                                         \
            if (local) d = PA_VMAX(VT, d, zero);                                                  \
            VT g = vgap[j];                                                                        \
            VT h = PA_VMAX(VT, PA_VMAX(VT, d, g), hgap);                                          \
            diag = hrow[j];                                                                        \
            hrow[j] = h;                                                                           \
            if (local) best = PA_VMAX(VT, best, h);                                              \
            VT hoe = h + vgoe;                                                                    \
            VT ge = g + vext, he = hgap + vext;                                                   \
            vgap[j] = PA_VMAX(VT, ge, hoe);                                                       \
            hgap = PA_VMAX(VT, he, hoe);                                                          \
        }                                                                                          \
        if (!local)                                                                                \
            for (int l = 0; l < L; ++l) if (ml[l] == i) res[l] = hrow[nl[l]][l];                  \
    }                                                                                              \
    for (int l = 0; l < lanes; ++l) {                                                             \
        if (local) res[l] = (ml[l] == 0 || nl[l] == 0) ? INT32_MIN : best[l];                    \
        x->scores[ids[l]] = res[l];                                                               \
    }                                                                                              \
    return PA_ORACLE_OK;                                                                          \
}

PA_SIMD_BATCH(simd_batch16, v8s, int16_t, 8, INT16_MIN)
PA_SIMD_BATCH(simd_batch32, v4i, int32_t, 4, INT32_MIN)

/* Code of a byte in the byte-lane mode: A C G T -> 0..3; a pair qualifies only when all of
 * its bytes are one of them, so equal codes are equal bytes, as the raw comparison of
 * score_model_unitary::score (score_model/score_model_unitary.hpp:52-59) requires. */
static inline int acgt_code(uint8_t b)
{
    return b == 'A' ? 0 : b == 'C' ? 1 : b == 'G' ? 2 : b == 'T' ? 3 : -1;
}

/* Local alignment in 16 unsigned-byte lanes.  A cell holds its true score (local scores are
 * >= 0).  The subtractions are floored at 0: max(x, c) - c.  For H that is the local clamp of
 * the diagonal term (dp_matrix_local.hpp:39-47); for the gap values it cannot change any H,
 * because H is itself >= 0 (max(g, 0) - ext and g - ext lead to the same maxima with a value
 * >= 0).  Additions of the match score cannot wrap while every value is <= 255 - match: the
 * first cell that would exceed that bound is computed from smaller inputs without wrapping, so
 * a lane whose best score stays <= 255 - match is exact and every other lane is redone.
 * Padding codes (0xfe in sequence1, 0xff in sequence2) never match, so padded cells only
 * lose score and never raise a lane's best. */
/* The batch's DP (pa_oracle_bytes.cpp): sequence codes in, each lane's best score out. */
void pa_oracle_byte_dp(const v16u *qvec, const v16u *tvec, v16u *hrow, v16u *vgap, uint64_t mmax, uint64_t nmax,
                       uint8_t match, uint8_t mis, uint8_t goe, uint8_t ext, v16u *best_out);

static int simd_batch8(simd_ctx *x, const uint32_t *ids, int lanes, v16u *qvec, v16u *tvec, v16u *hrow, v16u *vgap,
                       size_t cap_n)
{
    enum { L = 16 };
    const pa_oracle_cfg *c = x->cfg;
    uint64_t mmax = 0, nmax = 0, ml[L], nl[L];
    for (int l = 0; l < L; ++l) {
        uint32_t k = ids[l < lanes ? l : 0];
        ml[l] = x->off1[k + 1] - x->off1[k];
        nl[l] = x->off2[k + 1] - x->off2[k];
        if (ml[l] > mmax) mmax = ml[l];
        if (nl[l] > nmax) nmax = nl[l];
    }
    if (nmax + 1 > cap_n || mmax + 1 > cap_n) return PA_ORACLE_ENOMEM;
    for (int l = 0; l < L; ++l) {
        uint32_t k = ids[l < lanes ? l : 0];
        const uint8_t *a = x->s1 + x->off1[k], *b = x->s2 + x->off2[k];
        for (uint64_t i = 0; i < mmax; ++i) qvec[i][l] = (uint8_t)(i < ml[l] ? acgt_code(a[i]) : 0xfe);
        for (uint64_t j = 0; j < nmax; ++j) tvec[j][l] = (uint8_t)(j < nl[l] ? acgt_code(b[j]) : 0xff);
    }
    v16u best;
    pa_oracle_byte_dp(qvec, tvec, hrow, vgap, mmax, nmax, (uint8_t)c->match, (uint8_t)(-c->mismatch),
                      (uint8_t)(-(c->gap_open + c->gap_extension)), (uint8_t)(-c->gap_extension), &best);
    const int limit = 255 - c->match;
    for (int l = 0; l < lanes; ++l) {
        if ((int)best[l] > limit) x->redo[ids[l]] = 1;
        else x->scores[ids[l]] = (ml[l] == 0 || nl[l] == 0) ? INT32_MIN : (int32_t)best[l];
    }
    return PA_ORACLE_OK;
}

/* Workers pull batches of the lane count from a shared counter; each keeps its buffers. */
#define PA_SIMD_WORKER(FN, BATCH, VT, L)                                                           \
static void *FN(void *p)                                                                           \
{                                                                                                  \
    simd_ctx *x = (simd_ctx *)p;                                                                  \
    size_t cap_n = 0;                                                                              \
    VT *qvec = NULL, *tvec = NULL, *hrow = NULL, *vgap = NULL;                                    \
    for (;;) {                                                                                     \
        pthread_mutex_lock(&x->lock);                                                             \
        uint64_t b = x->next_batch++;                                                             \
        int rc_seen = x->rc;                                                                       \
        pthread_mutex_unlock(&x->lock);                                                           \
        uint64_t first = b * L;                                                                    \
        if (rc_seen || first >= x->n_pairs) break;                                                \
        int lanes = (int)((x->n_pairs - first) < L ? (x->n_pairs - first) : L);                  \
        const uint32_t *ids = x->order + first;                                                   \
        uint64_t mmax = 0, nmax = 0;                                                              \
        for (int l = 0; l < lanes; ++l) {                                                         \
            uint64_t m = x->off1[ids[l] + 1] - x->off1[ids[l]], n = x->off2[ids[l] + 1] - x->off2[ids[l]]; \
            if (m > mmax) mmax = m;                                                               \
            if (n > nmax) nmax = n;                                                               \
        }                                                                                          \
        if (nmax + 1 > cap_n || mmax + 1 > cap_n) {                                               \
            cap_n = (nmax > mmax ? nmax : mmax) + 1;                                              \
            free(qvec); free(tvec); free(hrow); free(vgap);                                       \
            qvec = (VT *)aligned_alloc(16, cap_n * sizeof(VT));                                   \
            tvec = (VT *)aligned_alloc(16, cap_n * sizeof(VT));                                   \
            hrow = (VT *)aligned_alloc(16, cap_n * sizeof(VT));                                   \
            vgap = (VT *)aligned_alloc(16, cap_n * sizeof(VT));                                   \
            if (!qvec || !tvec || !hrow || !vgap) {                                               \
                pthread_mutex_lock(&x->lock); x->rc = PA_ORACLE_ENOMEM; pthread_mutex_unlock(&x->lock); \
                break;                                                                             \
            }                                                                                      \
        }                                                                                          \
        int rc = BATCH(x, ids, lanes, qvec, tvec, hrow, vgap, cap_n);                            \
        if (rc) { pthread_mutex_lock(&x->lock); x->rc = rc; pthread_mutex_unlock(&x->lock); break; } \
    }                                                                                              \
    free(qvec); free(tvec); free(hrow); free(vgap);                                               \
    return NULL;                                                                                   \
}

PA_SIMD_WORKER(simd_worker16, simd_batch16, v8s, 8)
PA_SIMD_WORKER(simd_worker32, simd_batch32, v4i, 4)
PA_SIMD_WORKER(simd_worker8, simd_batch8, v16u, 16)

static const uint64_t *g_sort_off1, *g_sort_off2;
static int cmp_shape(const void *pa, const void *pb)
{
    uint32_t a = *(const uint32_t *)pa, b = *(const uint32_t *)pb;
    uint64_t ma = g_sort_off1[a + 1] - g_sort_off1[a], mb = g_sort_off1[b + 1] - g_sort_off1[b];
    uint64_t na = g_sort_off2[a + 1] - g_sort_off2[a], nb = g_sort_off2[b + 1] - g_sort_off2[b];
    if (na != nb) return na < nb ? -1 : 1;
    if (ma != mb) return ma < mb ? -1 : 1;
    return a < b ? -1 : (a > b);
}

/* Worst |value| a lane can see for this pair; mirrors the overflow guard a caller of the
 * reference's int16 / int32 SIMD models must respect. */
static int64_t lane_bound(const pa_oracle_cfg *c, uint64_t m, uint64_t n)
{
    int64_t a = llabs((int64_t)c->match), b = llabs((int64_t)c->mismatch);
    int64_t o = llabs((int64_t)c->gap_open), e = llabs((int64_t)c->gap_extension);
    int64_t s = a > b ? a : b;
    return s * (int64_t)(m < n ? m : n) + 2 * o + e * (int64_t)(m + n + 2) + o + e;
}

static int run_simd(simd_ctx *x, void *(*worker)(void *), int nthreads)
{
    pthread_mutex_init(&x->lock, NULL);
    pthread_t *th = (pthread_t *)calloc((size_t)nthreads, sizeof(pthread_t));
    if (!th) { pthread_mutex_destroy(&x->lock); return PA_ORACLE_ENOMEM; }
    for (int t = 1; t < nthreads; ++t) pthread_create(&th[t], NULL, worker, x);
    worker(x);
    for (int t = 1; t < nthreads; ++t) pthread_join(th[t], NULL);
    free(th);
    pthread_mutex_destroy(&x->lock);
    return x->rc;
}

/* The byte-lane mode applies to local alignment with scores that fit a byte; per pair, when
 * both sequences are all A/C/G/T. */
static int byte_lanes_apply(const pa_oracle_cfg *c)
{
    const int64_t goe = -(int64_t)c->gap_open - c->gap_extension, ext = -(int64_t)c->gap_extension;
    return c->local && c->match > 0 && c->match <= 127 && c->mismatch <= 0 && c->mismatch >= -255 && goe >= 0 &&
           goe <= 255 && ext >= 0 && ext <= 255;
}

static int pair_is_acgt(const uint8_t *s1, uint64_t m, const uint8_t *s2, uint64_t n)
{
    for (uint64_t i = 0; i < m; ++i) if (acgt_code(s1[i]) < 0) return 0;
    for (uint64_t j = 0; j < n; ++j) if (acgt_code(s2[j]) < 0) return 0;
    return 1;
}

int pa_oracle_simd_batch_lanes(const pa_oracle_cfg *c, const uint8_t *s1, const uint64_t *off1,
                               const uint8_t *s2, const uint64_t *off2, uint64_t n_pairs,
                               int32_t *scores, int nthreads, int byte_lanes, uint64_t counts[3])
{
    if (!c || !scores || (n_pairs && (!off1 || !off2))) return PA_ORACLE_EINVAL;
    if (c->local == 0 && (c->last_column_free || c->last_row_free)) return PA_ORACLE_EINVAL;
    if (c->dim) return PA_ORACLE_EINVAL;                /* the SIMD port scores unitary only */
    if (counts) counts[0] = counts[1] = counts[2] = 0;
    if (nthreads < 1) nthreads = 1;
    uint8_t *redo = NULL;
    const int use8 = byte_lanes && byte_lanes_apply(c) && n_pairs;
    if (use8) {
        /* byte lanes first; the pairs they cannot finish fall through to the wider lanes */
        uint32_t *order8 = (uint32_t *)malloc(sizeof(uint32_t) * n_pairs);
        redo = (uint8_t *)calloc(n_pairs, 1);
        if (!order8 || !redo) { free(order8); free(redo); return PA_ORACLE_ENOMEM; }
        uint64_t n8 = 0;
        for (uint64_t k = 0; k < n_pairs; ++k) {
            const uint64_t m = off1[k + 1] - off1[k], n = off2[k + 1] - off2[k];
            if (pair_is_acgt(s1 + off1[k], m, s2 + off2[k], n)) order8[n8++] = (uint32_t)k;
            else redo[k] = 1;
        }
        g_sort_off1 = off1; g_sort_off2 = off2;
        qsort(order8, n8, sizeof(uint32_t), cmp_shape);
        simd_ctx x;
        memset(&x, 0, sizeof(x));
        x.cfg = c; x.s1 = s1; x.off1 = off1; x.s2 = s2; x.off2 = off2; x.scores = scores; x.redo = redo;
        x.order = order8; x.n_pairs = n8;
        int rc = n8 ? run_simd(&x, simd_worker8, nthreads) : PA_ORACLE_OK;
        free(order8);
        if (rc) { free(redo); return rc; }
        if (counts) for (uint64_t k = 0; k < n_pairs; ++k) counts[0] += !redo[k];
    }
    uint32_t *order = (uint32_t *)malloc(sizeof(uint32_t) * (n_pairs ? n_pairs : 1) * 2);
    if (!order) { free(redo); return PA_ORACLE_ENOMEM; }
    uint32_t *order32 = order + (n_pairs ? n_pairs : 1);
    uint64_t n16 = 0, n32 = 0;
    for (uint64_t k = 0; k < n_pairs; ++k) {
        if (redo && !redo[k]) continue;               /* finished in byte lanes */
        uint64_t m = off1[k + 1] - off1[k], n = off2[k + 1] - off2[k];
        const int64_t bound = lane_bound(c, m, n);
        if (bound < 32000) order[n16++] = (uint32_t)k;
        else if (bound < (1ll << 30)) order32[n32++] = (uint32_t)k;
        else {                                    /* too wide for int32 lanes: scalar int64 */
            int64_t sc, e1, e2;
            int rc = pa_oracle_align(c, s1 + off1[k], m, s2 + off2[k], n, &sc, &e1, &e2);
            if (rc) { free(order); free(redo); return rc; }
            scores[k] = (int32_t)sc;
        }
    }
    free(redo);
    if (counts) { counts[1] = n16; counts[2] = n32; }
    g_sort_off1 = off1; g_sort_off2 = off2;
    qsort(order, n16, sizeof(uint32_t), cmp_shape);
    qsort(order32, n32, sizeof(uint32_t), cmp_shape);
    simd_ctx x;
    memset(&x, 0, sizeof(x));
    x.cfg = c; x.s1 = s1; x.off1 = off1; x.s2 = s2; x.off2 = off2; x.scores = scores;
    x.order = order; x.n_pairs = n16;
    int rc = n16 ? run_simd(&x, simd_worker16, nthreads) : PA_ORACLE_OK;
    if (!rc && n32) {
        x.order = order32; x.n_pairs = n32; x.next_batch = 0; x.rc = 0;
        rc = run_simd(&x, simd_worker32, nthreads);
    }
    free(order);
    return rc;
}

/* All lane widths the port has (byte lanes where they apply). */
int pa_oracle_simd_batch(const pa_oracle_cfg *c, const uint8_t *s1, const uint64_t *off1,
                         const uint8_t *s2, const uint64_t *off2, uint64_t n_pairs,
                         int32_t *scores, int nthreads)
{
    return pa_oracle_simd_batch_lanes(c, s1, off1, s2, off2, n_pairs, scores, nthreads, 1, NULL);
}
