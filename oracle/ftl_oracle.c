/*
 * CPU oracle -- TEST INFRASTRUCTURE ONLY.  A plain-C restatement of the
 * reference's partition-tree sampler (vbharadwaj-bk/fast_tensor_leverage,
 * cpp_ext/partition_tree.hpp), used by tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg as the checker.  The product never links it.
 *
 * Storage differs from the reference only in layout: node Grams are packed
 * upper triangles (element (a,b), a <= b, at a*R - a*(a-1)/2 + b - a) instead
 * of a full R x R buffer whose lower triangle is left zero.  Arithmetic and
 * every decision follow the reference line by line (cited per function).
 * Its own results are pinned against the reference module built from the
 * reference sources (oracle/Makefile) by tests/test_oracle.py and
 * the committed fixtures in tests/golden/.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
    int64_t n, F, leaf_count, node_count, lfill_level, lfill_count, total_levels,
        nodes_upto_lfill, nodes_before_lfill, complete_level_offset;
} orc_geom;

/* PartitionTree constructor, partition_tree.hpp:83-105; log2_round_down,
 * common.h:21-33. */
static orc_geom geom_of(int64_t n, int64_t F) {
    orc_geom g;
    g.n = n;
    g.F = F;
    g.leaf_count = (n + F - 1) / F;
    g.node_count = 2 * g.leaf_count - 1;
    g.lfill_level = 0;
    g.lfill_count = 1;
    while (g.lfill_count * 2 <= g.leaf_count) {
        g.lfill_level++;
        g.lfill_count *= 2;
    }
    g.total_levels = g.node_count > g.lfill_count ? g.lfill_level + 1 : g.lfill_level;
    g.nodes_upto_lfill = g.lfill_count * 2 - 1;
    g.nodes_before_lfill = g.lfill_count - 1;
    g.complete_level_offset = g.nodes_before_lfill - (g.node_count - g.nodes_upto_lfill) / 2;
    return g;
}

void orc_geometry(int64_t n, int64_t F, int64_t *out) {
    orc_geom g = geom_of(n, F);
    memcpy(out, &g, sizeof(g));
}

/* is_leaf / leaf_idx, partition_tree.hpp:107-118. */
static int is_leaf(const orc_geom *g, int64_t c) { return 2 * c + 1 >= g->node_count; }
static int64_t leaf_idx(const orc_geom *g, int64_t c) {
    return c >= g->nodes_upto_lfill ? c - g->nodes_upto_lfill : c - g->complete_level_offset;
}

static inline int64_t pk(int a, int b, int R) { return (int64_t)a * R - (int64_t)a * (a - 1) / 2 + (b - a); }

/* build_tree, partition_tree.hpp:120-170: leaf i (heap c = node_count -
 * leaf_count + i) holds the upper triangle of U_blk^T U_blk over its
 * row_ct = min(F, n - idx*F) rows; then G[c] += G[2c+1] + G[2c+2] level by
 * level from the lowest filled level up. */
void orc_tree_build(const double *U, int64_t n, int R, int64_t F, double *G) {
    orc_geom g = geom_of(n, F);
    const int64_t P = (int64_t)R * (R + 1) / 2;
    const int64_t first_leaf = g.node_count - g.leaf_count;
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < g.node_count * P; e++) G[e] = 0.0;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < g.leaf_count; i++) {
        int64_t idx = leaf_idx(&g, first_leaf + i);
        int64_t row_ct = F < n - idx * F ? F : n - idx * F;
        double *Gn = G + (first_leaf + i) * P;
        for (int a = 0; a < R; a++)
            for (int b = a; b < R; b++) {
                double acc = 0.0;
                for (int64_t r = 0; r < row_ct; r++)
                    acc += U[(idx * F + r) * R + a] * U[(idx * F + r) * R + b];
                Gn[pk(a, b, R)] = acc;
            }
    }
    int64_t start = g.nodes_before_lfill, end = first_leaf;
    for (int64_t lvl = g.lfill_level; lvl >= 0; lvl--) {
#pragma omp parallel for schedule(static)
        for (int64_t c = start; c < end; c++)
            for (int64_t e = 0; e < P; e++)
                G[c * P + e] += G[(2 * c + 1) * P + e] + G[(2 * c + 2) * P + e];
        end = start;
        start = ((start + 1) / 2) - 1;
    }
}

/* multiply_matrices_against_provided, partition_tree.hpp:183-194 (the
 * unmultiplied copy is the caller's src). */
void orc_tree_scale(const double *src, double *dst, int64_t node_count, int R, const double *mat) {
    const int64_t P = (int64_t)R * (R + 1) / 2;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < node_count; i++)
        for (int64_t e = 0; e < P; e++) dst[i * P + e] = src[i * P + e] * mat[e];
}

/* x^T G x as the reference evaluates it: y = G x with G symmetric from its
 * upper triangle (cblas_dsymv, partition_tree.hpp:66-81; here the textbook
 * upper-triangle dsymv loop over the packed rows), then the sequential dot
 * product of batch_dot_product (:201-214). */
static double qform(const double *Gn, const double *x, int R, double *y) {
    for (int a = 0; a < R; a++) y[a] = 0.0;
    const double *row = Gn;
    for (int a = 0; a < R; a++) {
        const double xa = x[a];
        double acc = row[0] * xa;
        for (int b = a + 1; b < R; b++) {
            acc += row[b - a] * x[b];
            y[b] += row[b - a] * xa;
        }
        y[a] += acc;
        row += R - a;
    }
    double m = 0.0;
    for (int a = 0; a < R; a++) m += x[a] * y[a];
    return m;
}

/* PTSample_internal, partition_tree.hpp:232-405, one sample at a time.
 * margin[i] (optional) receives the smallest distance, in draw units, between
 * the draw and any cutoff it was compared with (tree levels and leaf scan):
 * a sample whose margin is below the rounding noise of the quadratic forms
 * may legitimately be decided differently by another summation order. */
void orc_pt_sample(const double *G, const double *U, int64_t n, int R, int64_t F, double *h,
                   const double *scaled_h, uint64_t *samples, const double *draws, int64_t J,
                   double *margin) {
    orc_geom g = geom_of(n, F);
    const int64_t P = (int64_t)R * (R + 1) / 2;
#pragma omp parallel
    {
        double *y = (double *)malloc(sizeof(double) * R);
        double *q = (double *)malloc(sizeof(double) * (F > 0 ? F : 1));
#pragma omp for schedule(dynamic, 64)
        for (int64_t i = 0; i < J; i++) {
            const double *x = scaled_h + i * R;
            const double draw = draws[i];
            int64_t c = 0;
            double low = 0.0, high = 1.0, mg = INFINITY;
            double m = qform(G, x, R, y);
            for (int64_t lvl = 0; lvl < g.lfill_level; lvl++) {
                double mL = qform(G + (2 * c + 1) * P, x, R, y);
                double cutoff = low + mL / m;
                if (fabs(draw - cutoff) < mg) mg = fabs(draw - cutoff);
                if (draw <= cutoff) {
                    c = 2 * c + 1;
                    high = cutoff;
                } else {
                    c = 2 * c + 2;
                    low = cutoff;
                }
            }
            if (!is_leaf(&g, c)) { /* tail level, :304-332 */
                double mL = qform(G + (2 * c + 1) * P, x, R, y);
                double cutoff = low + mL / m;
                if (fabs(draw - cutoff) < mg) mg = fabs(draw - cutoff);
                if (draw <= cutoff) {
                    c = 2 * c + 1;
                    high = cutoff;
                } else {
                    c = 2 * c + 2;
                    low = cutoff;
                }
            }
            int64_t idx = leaf_idx(&g, c);
            int64_t res = 0;
            if (F > 1) { /* leaf dgemv and scan, :336-392 */
                double frac = (draw - low) / (high - low);
                int64_t row_count = F < n - idx * F ? F : n - idx * F;
                for (int64_t r = 0; r < F; r++) {
                    double acc = 0.0;
                    if (r < row_count)
                        for (int b = 0; b < R; b++) acc += U[(idx * F + r) * R + b] * x[b];
                    q[r] = acc;
                }
                res = F - 1;
                double run = 0.0;
                for (int64_t r = 0; r < F; r++) {
                    double t = q[r] * q[r];
                    q[r] = run;
                    run += t;
                }
                for (int64_t r = 0; r < F; r++) q[r] /= run;
                for (int64_t r = 0; r < F - 1; r++) {
                    double d = fabs(frac - q[r + 1]) * (high - low);
                    if (d < mg) mg = d;
                }
                for (int64_t r = 0; r < F - 1; r++) {
                    if (frac < q[r + 1]) {
                        res = r;
                        break;
                    }
                }
                /* A selection past the end of a partial block (frac rounding to
                 * >= 1) would read past the factor in the reference; the last
                 * row of the block is taken instead. */
                if (res >= row_count) res = row_count - 1;
            }
            int64_t s = res + idx * F;
            samples[i] = (uint64_t)s;
            for (int b = 0; b < R; b++) h[i * R + b] *= U[s * R + b];
            if (margin) margin[i] = mg;
        }
        free(y);
        free(q);
    }
}

/* Philox4x32-10 (Salmon et al., SC'11): uniform #i = 53 bits of the first
 * two output words of counter (ctr + i), key = seed -- the in-kernel
 * generator of the product, restated for the checker. */
static void philox_block(uint64_t seed, uint64_t counter, uint32_t out[4]) {
    uint32_t c0 = (uint32_t)counter, c1 = (uint32_t)(counter >> 32), c2 = 0, c3 = 0;
    uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
    for (int r = 0; r < 10; r++) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
        uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        c1 = (uint32_t)p1;
        c3 = (uint32_t)p0;
        c0 = n0;
        c2 = n2;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

/* Full 4x32 counter / 2x32 key block, for the generator's known-answer test. */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3], k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; r++) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
        uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        c1 = (uint32_t)p1;
        c3 = (uint32_t)p0;
        c0 = n0;
        c2 = n2;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

void orc_philox_uniforms(uint64_t seed, uint64_t ctr, int64_t n, double *out) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) {
        uint32_t w[4];
        philox_block(seed, ctr + (uint64_t)i, w);
        uint64_t bits = ((uint64_t)(w[0] >> 5) << 26) | (uint64_t)(w[1] >> 6);
        out[i] = (double)bits * (1.0 / 9007199254740992.0);
    }
}

int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_set_num_threads(int n) {
#ifdef _OPENMP
    omp_set_num_threads(n);
#else
    (void)n;
#endif
}
