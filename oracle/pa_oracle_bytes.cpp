/*
 * pa_oracle_bytes.cpp -- inner loop of the CPU port's byte lanes (TEST INFRASTRUCTURE ONLY:
 * part of the oracle library, the timed CPU baseline; never part of the product path).
 *
 * One batch of 16 local alignments, one per unsigned-byte lane, as pa_oracle.c's
 * simd_batch8 prepares it (sequence codes, padding, borders).  C++ because its vector
 * conditional (a > b ? a : b) lowers to the ISAs' native byte max (SSE2 pmaxub, NEON umax),
 * which the C form (compare plus bit select) does not.  The recurrence is the reference's
 * compute_cell (affine/affine_dp_algorithm.hpp:133-156) with the local clamp
 * (matrix/dp_matrix_local.hpp:39-47); the floors are explained in pa_oracle.c.
 */
#include <cstdint>

typedef uint8_t v16u __attribute__((vector_size(16)));

static inline v16u vmax(v16u a, v16u b) { return a > b ? a : b; }

extern "C" void pa_oracle_byte_dp(const v16u *qvec, const v16u *tvec, v16u *hrow, v16u *vgap, uint64_t mmax,
                                  uint64_t nmax, uint8_t match, uint8_t mis, uint8_t goe, uint8_t ext, v16u *best_out)
{
    const v16u zero = {};
    const v16u vmatch = zero + match, vmis = zero + mis, vgoe = zero + goe, vext = zero + ext;
    v16u best = zero;
    for (uint64_t j = 0; j <= nmax; ++j) { hrow[j] = zero; vgap[j] = zero; }
    for (uint64_t i = 1; i <= mmax; ++i) {
        v16u hgap = zero, diag = zero;
        const v16u qa = qvec[i - 1];
        for (uint64_t j = 1; j <= nmax; ++j) {
            const v16u d = qa == tvec[j - 1] ? diag + vmatch : vmax(diag, vmis) - vmis;
            const v16u g = vgap[j];
            const v16u h = vmax(vmax(d, g), hgap);
            diag = hrow[j];
            hrow[j] = h;
            best = vmax(best, h);
            const v16u hoe = vmax(h, vgoe) - vgoe;
            vgap[j] = vmax(vmax(g, vext) - vext, hoe);
            hgap = vmax(vmax(hgap, vext) - vext, hoe);
        }
    }
    *best_out = best;
}
