/*
 * oracle.c -- CPU restatement of Starflood's force-and-step path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker, never the product): see oracle.h.
 *
 * Each routine restates the reference algorithm in this code's own words;
 * the comments cite the reference lines (src/<file>:<line>) whose arithmetic
 * is reproduced.  Association order of every floating-point expression is
 * the reference's, and the library is built with -ffp-contract=off, so the
 * FP32 build is bit-identical to the reference on the same inputs (this is
 * checked against the compiled reference by tests/test_oracle.py).
 */
#include "oracle.h"

#include <math.h>
#include <stddef.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

typedef orc_real R;

#if defined(ORC_IS_DOUBLE)
#define R_SQRT(x) sqrt(x)
#define R_EXP(x) exp(x)
#define R_POW(x, y) pow((x), (y))
#else
#define R_SQRT(x) sqrtf(x)
#define R_EXP(x) expf(x)
#define R_POW(x, y) powf((x), (y))
#endif

/* 2^-32 rounded down to the float below it (rng.h:9). */
static const double k_inv_u32 = 2.3283062977608182109179324470460414886474609375e-10;
/* common.h:24, common.h:29 (the latter holds pi^(3/2) despite its name). */
static const double k_inv_sqrt_pi = 0.56418958354775628694807945156077258584405062932900;
static const double k_pi_pow_1_5 = 5.56832799683170784528481798211883570201362439028324;

/* Compensated running sum (the Kahan idiom of gravity.c:521-533).  The
 * volatile temporaries keep the compiler from reassociating, as in the
 * reference. */
typedef struct { R s, c; } ksum;
static inline void ksum_add(ksum* k, R x) {
    const R y = x - k->c;
    volatile R t = k->s + y;
    volatile R z = t - k->s;
    k->c = z - y;
    k->s = t;
}
typedef struct { double s, c; } ksum64;
static inline void ksum64_add(ksum64* k, double x) {
    const double y = x - k->c;
    volatile double t = k->s + y;
    volatile double z = t - k->s;
    k->c = z - y;
    k->s = t;
}

int orc_real_size(void) { return (int)sizeof(R); }

int orc_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ---- rng.h:13-40: one round of the pcg4d hash (Jarzynski & Olano 2020). */
void orc_pcg4d(uint32_t s[4]) {
    uint32_t a = s[0] * 1664525u + 1013904223u;
    uint32_t b = s[1] * 1664525u + 1013904223u;
    uint32_t c = s[2] * 1664525u + 1013904223u;
    uint32_t d = s[3] * 1664525u + 1013904223u;
    a += b * d; b += c * a; c += a * b; d += b * c;
    a ^= a >> 16; b ^= b >> 16; c ^= c >> 16; d ^= d >> 16;
    a += b * d; b += c * a; c += a * b; d += b * c;
    s[0] = a; s[1] = b; s[2] = c; s[3] = d;
}

/* ---- simulation.c:245-277: mean distance from the origin, FP64 + Kahan. */
double orc_mean_radius(uint32_t n, const R* pos) {
    ksum64 acc = {0.0, 0.0};
    for (uint32_t i = 0; i < n; i++) {
        const double x = (double)pos[3u * i + 0u];
        const double y = (double)pos[3u * i + 1u];
        const double z = (double)pos[3u * i + 2u];
        ksum64_add(&acc, sqrt((x * x) + (y * y) + (z * z)));
    }
    return acc.s * (1.0 / (double)n);
}

/* ---- simulation.c:279-301: root cube = [-2r, 2r] shifted by r*j/2 per axis,
 * j in [-1, 1) from pcg4d seeded with the step number. */
void orc_root_bounds(uint32_t n, const R* pos, uint32_t step_number, R bounds[6]) {
    const double rbar = orc_mean_radius(n, pos);
    uint32_t h[4] = {0x638FE17Bu + step_number, 0xB10BDCE7u, 0x7B8ADB9Bu, 0xD8C5850Eu};
    orc_pcg4d(h);
    for (int a = 0; a < 3; a++) {
        const double j = 2.0 * (k_inv_u32 * (double)h[a]) - 1.0;
        bounds[a] = (R)(-2.000 * rbar + 0.5 * j * rbar);
        bounds[3 + a] = (R)(2.000 * rbar + 0.5 * j * rbar);
    }
}

/* ---- tree.c:74-318: build by inserting particles one at a time. */
static void node_clear(orc_node* nd, uint32_t parent) {
    memset(nd, 0, sizeof(*nd));
    nd->parent = parent;
}

int orc_tree_build(const orc_params* p, uint32_t n, const R* pos, const R* mas,
                   const R bounds[6], orc_node* nodes, uint32_t* num_nodes) {
    const uint32_t cap = p->leaf_cap;
    const uint32_t max_nodes = p->nodes_max;
    const int depth_max = (int)p->depth_max;
    uint32_t count = 1u;

    /* tree.c:85-107 purge, 112-115 root bounds */
    for (uint32_t i = 0; i < max_nodes; i++) node_clear(&nodes[i], 0u);
    for (int a = 0; a < 6; a++) nodes[0].bounds[a] = bounds[a];

    int status = 0;
    for (uint32_t idx = 0; idx < n && status == 0; idx++) {
        const R x[3] = {pos[3u * idx], pos[3u * idx + 1u], pos[3u * idx + 2u]};
        const R m = mas[idx];
        R lo[3] = {bounds[0], bounds[1], bounds[2]};
        R hi[3] = {bounds[3], bounds[4], bounds[5]};

        /* tree.c:141-146: particles outside the closed root cube are skipped */
        int outside = 0;
        for (int a = 0; a < 3; a++) outside |= (lo[a] > x[a]) | (x[a] > hi[a]);
        if (outside) continue;

        uint32_t cur = 0u;
        for (int depth = 0; depth <= depth_max; depth++) {
            orc_node* nd = &nodes[cur];
            const uint32_t before = nd->bodies;           /* tree.c:154-156 */
            nd->bodies = before + 1u;
            R mid[3];
            for (int a = 0; a < 3; a++) mid[a] = (R)0.5 * (lo[a] + hi[a]);  /* 203-207 */
            nd->params[0] += m * x[0];                    /* 210-213 */
            nd->params[1] += m * x[1];
            nd->params[2] += m * x[2];
            nd->params[3] += m;

            if (before < cap) {                           /* 216-219 */
                nd->branch[before] = idx;
                break;
            }
            if (before == cap) {                          /* 222-318: split */
                if (max_nodes <= count + 8u) { status = -1; break; }
                if (depth_max <= depth) { status = -1; break; }
                orc_node kids[8];
                for (int o = 0; o < 8; o++) {
                    node_clear(&kids[o], cur);
                    for (int a = 0; a < 3; a++) {
                        const int up = (o >> a) & 1;
                        kids[o].bounds[a] = up ? mid[a] : lo[a];
                        kids[o].bounds[3 + a] = up ? hi[a] : mid[a];
                    }
                }
                /* 273-304: the resident particles move down, in slot order,
                 * choosing the upper half only when strictly above mid. */
                for (uint32_t k = 0; k < cap; k++) {
                    const uint32_t q = nd->branch[k];
                    const R y[3] = {pos[3u * q], pos[3u * q + 1u], pos[3u * q + 2u]};
                    const R mq = mas[q];
                    const int o = (mid[0] < y[0] ? 1 : 0) + (mid[1] < y[1] ? 2 : 0) +
                                  (mid[2] < y[2] ? 4 : 0);
                    orc_node* kd = &kids[o];
                    kd->branch[kd->bodies] = q;
                    kd->bodies += 1u;
                    kd->params[0] += mq * y[0];
                    kd->params[1] += mq * y[1];
                    kd->params[2] += mq * y[2];
                    kd->params[3] += mq;
                }
                for (int o = 0; o < 8; o++) {             /* 307-317 */
                    nodes[count + (uint32_t)o] = kids[o];
                    nd->branch[o] = count + (uint32_t)o;
                }
                for (uint32_t k = 8; k < ORC_LEAF_MAX; k++) nd->branch[k] = 0u;
                count += 8u;
            }
            /* 326-338: the arriving particle picks the upper half when at or
             * above mid. */
            const int o = (mid[0] <= x[0] ? 1 : 0) + (mid[1] <= x[1] ? 2 : 0) +
                          (mid[2] <= x[2] ? 4 : 0);
            for (int a = 0; a < 3; a++) {
                if ((o >> a) & 1) lo[a] = mid[a]; else hi[a] = mid[a];
            }
            cur = nd->branch[o];
        }
    }
    *num_nodes = count;
    if (status != 0) return -1;   /* tree.c:179-189 leave COMs unnormalised */

    for (uint32_t i = 0; i < count; i++) {                /* tree.c:302-310 */
        const R w = nodes[i].params[3];
        const R inv = (R)0.0 < w ? (R)1.0 / w : (R)1.0;
        nodes[i].params[0] *= inv;
        nodes[i].params[1] *= inv;
        nodes[i].params[2] *= inv;
    }
    return 0;
}

/* ---- gravity.c:242-663: per-particle depth-first walk without a stack of
 * node ids: parent links plus the octant being visited at every depth. */
static void gravity_tree_impl(const orc_params* p, uint32_t n, const R* pos, const R* mas,
                              const orc_node* nodes, R* acc, R* pot, orc_walk_stats* stats, R* mag) {
    const uint32_t cap = p->leaf_cap;
    const R eps2 = (R)(p->eps * p->eps);
    const R theta = (R)p->theta;
    const R third = (R)(1.0 / 3.0);
    const R neg_g = (R)(-p->G);
    const int depth_max = (int)p->depth_max;
    const uint64_t iter_cap = 2ull * 8ull * (uint64_t)p->nodes_max;   /* 306 */

#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 256)
#endif
    for (int64_t ii = 0; ii < (int64_t)n; ii++) {
        const uint32_t i = (uint32_t)ii;
        const R ri[3] = {pos[3u * i], pos[3u * i + 1u], pos[3u * i + 2u]};
        const R mi = mas[i];
        ksum ax = {0, 0}, ay = {0, 0}, az = {0, 0}, ph = {0, 0};
        double tmag = 0.0;  /* sum of |term| (FP64), the scale of the sum's rounding */
        uint32_t n_int = 0u, n_open = 0u;

        int path[64];
        for (int d = 0; d < depth_max; d++) path[d] = -1;
        uint32_t at = 0u;
        int depth = 0;
        for (uint64_t it = 0; it < iter_cap && depth >= 0; it++) {
            const orc_node* nd = &nodes[at];
            const R* lo = &nd->bounds[0];
            const R* hi = &nd->bounds[3];
            if (nd->bodies == 0u) {                       /* 324-328 */
                at = nd->parent;
                depth--;
                continue;
            }
            if (nd->bodies > cap) {                       /* 331-461 */
                const int oct = path[depth];
                if (oct >= 7) {
                    at = nd->parent;
                    path[depth] = -1;
                    depth--;
                    continue;
                }
                if (oct >= 0) {
                    at = nd->branch[oct + 1];
                    path[depth] = oct + 1;
                    depth++;
                    continue;
                }
                /* 352-377: squared width over squared distance to the
                 * geometric centre of the cell. */
                n_open++;
                const R cx = (R)0.5 * (lo[0] + hi[0]);
                const R cy = (R)0.5 * (lo[1] + hi[1]);
                const R cz = (R)0.5 * (lo[2] + hi[2]);
                const R ox = cx - ri[0], oy = cy - ri[1], oz = cz - ri[2];
                const R d2 = (ox * ox) + (oy * oy) + (oz * oz);
                const R w = third * ((hi[0] - lo[0]) + (hi[1] - lo[1]) + (hi[2] - lo[2]));
                const R ratio = (R)0.0 < d2 ? (w * w) / d2 : (R)0.0;
                if (theta <= ratio) {                     /* 448-453 */
                    at = nd->branch[0];
                    path[depth] = 0;
                    depth++;
                    continue;
                }
            }
            /* 463-490: monopole, with particle i taken out when it lies in
             * the closed cell and the cell holds more than one body. */
            R cm[3] = {nd->params[0], nd->params[1], nd->params[2]};
            R mj = nd->params[3];
            if (lo[0] <= ri[0] && ri[0] <= hi[0] && lo[1] <= ri[1] && ri[1] <= hi[1] &&
                lo[2] <= ri[2] && ri[2] <= hi[2] && 1u < nd->bodies) {
                for (int a = 0; a < 3; a++) cm[a] *= mj;
                for (int a = 0; a < 3; a++) cm[a] -= mi * ri[a];
                mj -= mi;
                for (int a = 0; a < 3; a++) cm[a] *= (R)0.0 < mj ? (R)1.0 / mj : (R)1.0;
            }
            /* 493-548 */
            const R dx = ri[0] - cm[0], dy = ri[1] - cm[1], dz = ri[2] - cm[2];
            const R r2 = (dx * dx) + (dy * dy) + (dz * dz);
            const R inv2 = (R)1.0 / (r2 + eps2);
            const R inv1 = (R)1.0 / R_SQRT(r2 + eps2);
            const R phi = mj * inv1;
            if (p->kahan) {
                ksum_add(&ax, phi * inv2 * dx);
                ksum_add(&ay, phi * inv2 * dy);
                ksum_add(&az, phi * inv2 * dz);
                ksum_add(&ph, phi);
            } else {
                ax.s += phi * inv2 * dx;
                ay.s += phi * inv2 * dy;
                az.s += phi * inv2 * dz;
                ph.s += phi;
            }
            if (mag) tmag += (double)(phi * inv2) * sqrt((double)r2);
            n_int++;
            at = nd->parent;                              /* 577-578 */
            depth--;
        }
        acc[3u * i + 0u] = neg_g * mi * ax.s;             /* 656-659 */
        acc[3u * i + 1u] = neg_g * mi * ay.s;
        acc[3u * i + 2u] = neg_g * mi * az.s;
        pot[i] = neg_g * ph.s;
        if (stats) {
            stats[i].interactions = n_int;
            stats[i].opening_tests = n_open;
        }
        if (mag) mag[i] = (R)(fabs((double)neg_g) * fabs((double)mi) * tmag);
    }
}

void orc_gravity_tree(const orc_params* p, uint32_t n, const R* pos, const R* mas,
                      const orc_node* nodes, R* acc, R* pot, orc_walk_stats* stats) {
    gravity_tree_impl(p, n, pos, mas, nodes, acc, pot, stats, NULL);
}

/* The same walk, also returning per body G m_i sum_k |F_k|: the sum of the
 * magnitudes of the terms whose vector sum is acc_i (test infrastructure:
 * the scale against which a body's rounding error is judged when its terms
 * cancel). */
void orc_gravity_tree_mag(const orc_params* p, uint32_t n, const R* pos, const R* mas,
                          const orc_node* nodes, R* acc, R* pot, orc_walk_stats* stats, R* mag) {
    gravity_tree_impl(p, n, pos, mas, nodes, acc, pot, stats, mag);
}

/* ---- gravity.c:666-819: every j, including j == i. */
void orc_gravity_pp(const orc_params* p, uint32_t n, const R* pos, const R* mas,
                    R* acc, R* pot) {
    const R eps2 = (R)(p->eps * p->eps);
    const R neg_g = (R)(-p->G);
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 256)
#endif
    for (int64_t ii = 0; ii < (int64_t)n; ii++) {
        const uint32_t i = (uint32_t)ii;
        const R mi = mas[i];
        const R xi = pos[3u * i], yi = pos[3u * i + 1u], zi = pos[3u * i + 2u];
        ksum ax = {0, 0}, ay = {0, 0}, az = {0, 0}, ph = {0, 0};
        for (uint32_t j = 0; j < n; j++) {
            const R dx = xi - pos[3u * j];
            const R dy = yi - pos[3u * j + 1u];
            const R dz = zi - pos[3u * j + 2u];
            const R r2 = (dx * dx) + (dy * dy) + (dz * dz);
            const R inv2 = (R)1.0 / (r2 + eps2);
            const R inv1 = (R)1.0 / R_SQRT(r2 + eps2);
            const R phi = mas[j] * inv1;
            if (p->kahan) {
                ksum_add(&ax, phi * inv2 * dx);
                ksum_add(&ay, phi * inv2 * dy);
                ksum_add(&az, phi * inv2 * dz);
                ksum_add(&ph, phi);
            } else {
                ax.s += phi * inv2 * dx;
                ay.s += phi * inv2 * dy;
                az.s += phi * inv2 * dz;
                ph.s += phi;
            }
        }
        acc[3u * i + 0u] = neg_g * mi * ax.s;
        acc[3u * i + 1u] = neg_g * mi * ay.s;
        acc[3u * i + 2u] = neg_g * mi * az.s;
        pot[i] = neg_g * ph.s;
    }
}

/* The same sums for the bodies idx[0..ni) only, over all n bodies j (a
 * seeded subsample of a workload too large for all pairs); outputs are
 * indexed like idx. */
void orc_gravity_pp_subset(const orc_params* p, uint32_t n, const R* pos, const R* mas, uint32_t ni,
                           const uint32_t* idx, R* acc, R* pot, R* mag) {
    const R eps2 = (R)(p->eps * p->eps);
    const R neg_g = (R)(-p->G);
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 4)
#endif
    for (int64_t kk = 0; kk < (int64_t)ni; kk++) {
        const uint32_t i = idx[kk];
        const R mi = mas[i];
        const R xi = pos[3u * i], yi = pos[3u * i + 1u], zi = pos[3u * i + 2u];
        ksum ax = {0, 0}, ay = {0, 0}, az = {0, 0}, ph = {0, 0};
        double tmag = 0.0;
        for (uint32_t j = 0; j < n; j++) {
            const R dx = xi - pos[3u * j];
            const R dy = yi - pos[3u * j + 1u];
            const R dz = zi - pos[3u * j + 2u];
            const R r2 = (dx * dx) + (dy * dy) + (dz * dz);
            const R inv2 = (R)1.0 / (r2 + eps2);
            const R inv1 = (R)1.0 / R_SQRT(r2 + eps2);
            const R phi = mas[j] * inv1;
            ksum_add(&ax, phi * inv2 * dx);
            ksum_add(&ay, phi * inv2 * dy);
            ksum_add(&az, phi * inv2 * dz);
            ksum_add(&ph, phi);
            if (mag) tmag += (double)(phi * inv2) * sqrt((double)r2);
        }
        acc[3u * kk + 0u] = neg_g * mi * ax.s;
        acc[3u * kk + 1u] = neg_g * mi * ay.s;
        acc[3u * kk + 2u] = neg_g * mi * az.s;
        pot[kk] = neg_g * ph.s;
        if (mag) mag[kk] = (R)(fabs((double)neg_g) * fabs((double)mi) * tmag);
    }
}

/* ---- sph.c:14-282: Gaussian kernel W = (1/(sqrt(pi) h))^3 exp(-r^2/h^2),
 * density over all pairs, polytrope P = (0.1 rho)^2, momentum over pairs with
 * r^2 <= 1. */
void orc_sph_reference(const orc_params* p, uint32_t n, const R* pos, const R* mas,
                       const R* rad, R* rho, R* prs, R* acc, uint32_t* nbr) {
    (void)p;
    const R inv_sqrt_pi = (R)k_inv_sqrt_pi;
    const R pi_1_5 = (R)k_pi_pow_1_5;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 256)
#endif
    for (int64_t ii = 0; ii < (int64_t)n; ii++) {          /* sph.c:35-145 */
        const uint32_t i = (uint32_t)ii;
        const R hi = rad[i];
        const R xi = pos[3u * i], yi = pos[3u * i + 1u], zi = pos[3u * i + 2u];
        ksum s = {0, 0};
        for (uint32_t j = 0; j < n; j++) {
            const R hj = rad[j];
            const R dx = xi - pos[3u * j];
            const R dy = yi - pos[3u * j + 1u];
            const R dz = zi - pos[3u * j + 2u];
            const R r2 = (dx * dx) + (dy * dy) + (dz * dz);
            const R ai = inv_sqrt_pi / hi;
            const R aj = inv_sqrt_pi / hj;
            const R wi = (ai * ai * ai) * R_EXP(-r2 / (hi * hi));
            const R wj = (aj * aj * aj) * R_EXP(-r2 / (hj * hj));
            ksum_add(&s, (R)0.5 * (wi + wj) * mas[j]);
        }
        rho[i] = s.s;
    }
    const R eos_k = (R)0.100;                               /* sph.c:148-159 */
    const R eos_e = (R)((1.0 / 1.0) + 1.0);
    for (uint32_t i = 0; i < n; i++) prs[i] = R_POW(eos_k * rho[i], eos_e);

#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 256)
#endif
    for (int64_t ii = 0; ii < (int64_t)n; ii++) {          /* sph.c:172-277 */
        const uint32_t i = (uint32_t)ii;
        const R mi = mas[i];
        const R hi = rad[i];
        const R xi = pos[3u * i], yi = pos[3u * i + 1u], zi = pos[3u * i + 2u];
        const R rhoi2 = rho[i] * rho[i];
        const R ci = (R)0.0 < rhoi2 ? prs[i] / rhoi2 : (R)0.0;
        ksum sx = {0, 0}, sy = {0, 0}, sz = {0, 0};
        uint32_t count = 0u;
        for (uint32_t j = 0; j < n; j++) {
            const R hj = rad[j];
            const R dx = xi - pos[3u * j];
            const R dy = yi - pos[3u * j + 1u];
            const R dz = zi - pos[3u * j + 2u];
            const R rhoj2 = rho[j] * rho[j];
            const R cj = (R)0.0 < rhoj2 ? prs[j] / rhoj2 : (R)0.0;
            const R r2 = (dx * dx) + (dy * dy) + (dz * dz);
            if (r2 > (R)(1.000 * 1.000)) continue;          /* sph.c:231 */
            count++;
            const R ni = (R)-2.0 * R_EXP(-r2 / (hi * hi)) / (pi_1_5 * hi * hi * hi * hi * hi);
            const R nj = (R)-2.0 * R_EXP(-r2 / (hj * hj)) / (pi_1_5 * hj * hj * hj * hj * hj);
            const R g = (R)0.5 * (ni + nj);
            ksum_add(&sx, (ci + cj) * (g * dx));
            ksum_add(&sy, (ci + cj) * (g * dy));
            ksum_add(&sz, (ci + cj) * (g * dz));
        }
        acc[3u * i + 0u] += -mi * sx.s;
        acc[3u * i + 1u] += -mi * sy.s;
        acc[3u * i + 2u] += -mi * sz.s;
        if (nbr) nbr[i] = count;
    }
}

/* ---- simulation.h:17-51: SIM_DOF = 13, or 16 with SPH. */
uint32_t orc_sim_dof(const orc_params* p) { return p->use_sph ? 16u : 13u; }

/* slab offsets (simulation.c:33-53) */
#define SLAB(s, k) ((s)->mem + (size_t)(s)->N * (size_t)(k))

int orc_sim_solv(const orc_params* p, orc_sim* s) {
    const uint32_t n = s->N;
    R* pos = SLAB(s, 0);
    R* acc = SLAB(s, 6);
    R* mas = SLAB(s, 9);
    R* pot = SLAB(s, 10);
    int status = 0;
    if (p->use_tree) {                                      /* simulation.c:244-325 */
        orc_root_bounds(n, pos, s->step_number, s->bounds);
        s->tree_status = orc_tree_build(p, n, pos, mas, s->bounds, s->nodes, &s->num_nodes);
        /* the reference ignores the build status (simulation.c:312) */
        orc_gravity_tree(p, n, pos, mas, s->nodes, acc, pot, NULL);
    } else {                                                /* simulation.c:329 */
        orc_gravity_pp(p, n, pos, mas, acc, pot);
    }
    if (p->use_sph) {                                       /* simulation.c:338 */
        orc_sph_reference(p, n, pos, mas, SLAB(s, 13), SLAB(s, 14), SLAB(s, 15), acc, NULL);
    }
    return status;
}

int orc_sim_step(const orc_params* p, orc_sim* s, double* T, double* V) {
    const uint32_t n = s->N;
    R* pos = SLAB(s, 0);
    R* vel = SLAB(s, 3);
    R* acc = SLAB(s, 6);
    R* mas = SLAB(s, 9);
    R* pot = SLAB(s, 10);
    R* ken = SLAB(s, 11);
    R* pen = SLAB(s, 12);
    const R dt = (R)p->dt;
    const R half_dt = (R)0.5 * dt;

    for (uint32_t k = 0; k < 3u * n; k++) vel[k] += half_dt * acc[k];   /* 381-383 */
    for (uint32_t k = 0; k < 3u * n; k++) pos[k] += dt * vel[k];        /* 393-395 */
    const int status = orc_sim_solv(p, s);                               /* 406-413 */
    for (uint32_t k = 0; k < 3u * n; k++) vel[k] += half_dt * acc[k];   /* 423-425 */

    for (uint32_t i = 0; i < n; i++) {                                   /* 434-446 */
        const R vx = vel[3u * i], vy = vel[3u * i + 1u], vz = vel[3u * i + 2u];
        const R v2 = (vx * vx) + (vy * vy) + (vz * vz);
        ken[i] = (R)0.5 * mas[i] * v2;
    }
    for (uint32_t i = 0; i < n; i++) pen[i] = mas[i] * pot[i];          /* 449-451 */

    ksum64 tk = {0.0, 0.0}, vk = {0.0, 0.0};                             /* 455-497 */
    for (uint32_t i = 0; i < n; i++) ksum64_add(&tk, (double)ken[i]);
    for (uint32_t i = 0; i < n; i++) ksum64_add(&vk, (double)pen[i]);
    if (T) *T = tk.s;
    if (V) *V = vk.s;
    return status;
}

/* ---- cubic-spline SPH (no reference counterpart; FP64 oracle) --------------
 * Kernel: Monaghan & Lattanzio (1985) M4 cubic spline in 3-D, support 2h,
 *   W(r,h) = 1/(pi h^3) * (1 - 1.5 q^2 + 0.75 q^3)  0 <= q < 1
 *                        * 0.25 (2 - q)^3            1 <= q < 2,  q = r/h
 * symmetrised W_ij = (W(r,h_i) + W(r,h_j))/2 when smoothing lengths differ.
 * Equation of state P = (gamma - 1) rho u, sound speed c = sqrt(gamma P/rho).
 * Monaghan (1992) viscosity Pi_ij = (-alpha cbar mu + beta mu^2)/rhobar for
 * v_ij.r_ij < 0, mu = h v_ij.r_ij/(r^2 + 0.01 h^2), h = (h_i + h_j)/2.
 *   dv_i/dt = -sum_j m_j (P_i/rho_i^2 + P_j/rho_j^2 + Pi_ij) grad_i W_ij
 *   du_i/dt =  sum_j m_j (P_i/rho_i^2 + Pi_ij/2) v_ij . grad_i W_ij
 * Neighbours: j with fl32((dx^2 + dy^2) + dz^2) < fl32((2 max(h_i,h_j))^2),
 * dx = fl32(x_i - x_j), the FP32 decision the GPU makes; physics in FP64. */
static double cubic_w(double r, double h) {
    const double q = r / h;
    const double s = 1.0 / (3.14159265358979323846 * h * h * h);
    if (q < 1.0) return s * (1.0 - 1.5 * q * q + 0.75 * q * q * q);
    if (q < 2.0) return s * 0.25 * (2.0 - q) * (2.0 - q) * (2.0 - q);
    return 0.0;
}
static double cubic_dw(double r, double h) {  /* dW/dr */
    const double q = r / h;
    const double s = 1.0 / (3.14159265358979323846 * h * h * h * h);
    if (q < 1.0) return s * (-3.0 * q + 2.25 * q * q);
    if (q < 2.0) return s * (-0.75 * (2.0 - q) * (2.0 - q));
    return 0.0;
}
static int cubic_neighbour(const float* pos, const float* rad, uint32_t i, uint32_t j) {
    volatile float dx = pos[3u * i] - pos[3u * j];
    volatile float dy = pos[3u * i + 1u] - pos[3u * j + 1u];
    volatile float dz = pos[3u * i + 2u] - pos[3u * j + 2u];
    volatile float xx = dx * dx, yy = dy * dy, zz = dz * dz;
    volatile float r2 = (xx + yy) + zz;
    volatile float hm = rad[i] > rad[j] ? rad[i] : rad[j];
    volatile float s = 2.0f * hm;
    volatile float s2 = s * s;
    return r2 < s2;
}

void orc_sph_cubic(uint32_t n, const float* pos, const float* vel, const float* mas, const float* rad,
                   const float* u, double gamma, double alpha, double beta, double* rho, double* prs,
                   double* acc, double* dudt, uint32_t* nbr) {
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 64)
#endif
    for (int64_t ii = 0; ii < (int64_t)n; ii++) {
        const uint32_t i = (uint32_t)ii;
        double s = 0.0;
        uint32_t cnt = 0;
        for (uint32_t j = 0; j < n; j++) {
            if (!cubic_neighbour(pos, rad, i, j)) continue;
            cnt++;
            const double dx = (double)pos[3u * i] - pos[3u * j];
            const double dy = (double)pos[3u * i + 1u] - pos[3u * j + 1u];
            const double dz = (double)pos[3u * i + 2u] - pos[3u * j + 2u];
            const double r = sqrt(dx * dx + dy * dy + dz * dz);
            s += (double)mas[j] * 0.5 * (cubic_w(r, rad[i]) + cubic_w(r, rad[j]));
        }
        rho[i] = s;
        prs[i] = (gamma - 1.0) * s * (double)u[i];
        if (nbr) nbr[i] = cnt;
    }
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 64)
#endif
    for (int64_t ii = 0; ii < (int64_t)n; ii++) {
        const uint32_t i = (uint32_t)ii;
        const double ci = sqrt(gamma * (gamma - 1.0) * (double)u[i]);
        const double pi_ = rho[i] > 0.0 ? prs[i] / (rho[i] * rho[i]) : 0.0;
        double ax = 0.0, ay = 0.0, az = 0.0, du = 0.0;
        for (uint32_t j = 0; j < n; j++) {
            if (j == i || !cubic_neighbour(pos, rad, i, j)) continue;
            const double dx = (double)pos[3u * i] - pos[3u * j];
            const double dy = (double)pos[3u * i + 1u] - pos[3u * j + 1u];
            const double dz = (double)pos[3u * i + 2u] - pos[3u * j + 2u];
            const double r2 = dx * dx + dy * dy + dz * dz;
            const double r = sqrt(r2);
            if (!(r > 0.0)) continue;
            const double g = 0.5 * (cubic_dw(r, rad[i]) + cubic_dw(r, rad[j])) / r;  /* grad W = g r_ij */
            const double vx = (double)vel[3u * i] - vel[3u * j];
            const double vy = (double)vel[3u * i + 1u] - vel[3u * j + 1u];
            const double vz = (double)vel[3u * i + 2u] - vel[3u * j + 2u];
            const double vr = vx * dx + vy * dy + vz * dz;
            const double pj = rho[j] > 0.0 ? prs[j] / (rho[j] * rho[j]) : 0.0;
            double visc = 0.0;
            if (vr < 0.0) {
                const double h = 0.5 * ((double)rad[i] + rad[j]);
                const double mu = h * vr / (r2 + 0.01 * h * h);
                const double cj = sqrt(gamma * (gamma - 1.0) * (double)u[j]);
                const double cbar = 0.5 * (ci + cj), rbar = 0.5 * (rho[i] + rho[j]);
                visc = (-alpha * cbar * mu + beta * mu * mu) / rbar;
            }
            const double f = (double)mas[j] * (pi_ + pj + visc) * g;
            ax -= f * dx;
            ay -= f * dy;
            az -= f * dz;
            du += (double)mas[j] * (pi_ + 0.5 * visc) * g * vr;
        }
        acc[3u * i] = ax;
        acc[3u * i + 1u] = ay;
        acc[3u * i + 2u] = az;
        dudt[i] = du;
    }
}

/* ---- visualization.c:258-740: vis_draw, the atomic splat rasteriser ------- */
#define ORC_TAU 6.28318530717958647692528676655900576839433879875021

/* x86 float->int: out of range and NaN give INT_MIN (the reference's (int)). */
static int vis_to_int(float v) { return (v >= -2147483648.0f && v < 2147483648.0f) ? (int)v : INT32_MIN; }

void orc_vis_draw(uint32_t n, const float* pos, const float* vel, const float* pot, uint32_t step,
                  double timestep, uint32_t sizex, uint32_t sizey, uint32_t samples, double exposure,
                  double ortho_scale, int autoscale, int tonemap, int32_t* accum, float* render) {
    /* mean radius, FP64 Kahan in index order (visualization.c:276-305) */
    double sum = 0.0, comp = 0.0;
    for (uint32_t i = 0; i < n; i++) {
        const double x = pos[3u * i], y = pos[3u * i + 1u], z = pos[3u * i + 2u];
        const double r = sqrt((x * x) + (y * y) + (z * z));
        const double yk = r - comp;
        volatile double t = sum + yk;
        volatile double d = t - sum;
        comp = d - yk;
        sum = t;
    }
    const double mean = sum * (1.0 / (double)n);
    /* camera (visualization.c:318-480): model rotation, orthographic scale */
    const float time = (float)(timestep * (double)step);
    float alp = 0.0f, bet = (float)ORC_TAU * 0.1250f, gam = (float)ORC_TAU * 0.0625f;
    alp += (float)ORC_TAU * 1.000e-4f * time;
    bet += (float)ORC_TAU * 1.000e-4f * time;
    gam += (float)ORC_TAU * 1.000e-4f * time;
    const float ca = cosf(alp), sa = sinf(alp), cb = cosf(bet), sb = sinf(bet), cg = cosf(gam), sg = sinf(gam);
    const float M[16] = {ca * cb, ca * sb * sg - sa * cg, ca * sb * cg + sa * sg, 0.0f,
                         sa * cb, sa * sb * sg + ca * cg, sa * sb * cg - ca * sg, 0.0f,
                         -sb,     cb * sg,                cb * cg,                0.0f,
                         0.0f,    0.0f,                   0.0f,                   1.0f};
    float scale = (float)exp2(ortho_scale);
    if (autoscale) scale *= (float)(1.0 / mean);
    /* P (V M) with V = I and P = diag(scale, scale, scale, 1): every term
     * but one of each product is an exact zero */
    float MVP[16];
    for (int k = 0; k < 16; k++) MVP[k] = (k < 12) ? scale * M[k] : M[k];
    memset(accum, 0, sizeof(int32_t) * 4u * (size_t)sizex * sizey);
    const float half_x = 0.5f * (float)sizex, half_y = 0.5f * (float)sizey;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 256)
#endif
    for (uint32_t i = 0; i < n; i++) {
        const float x[4] = {pos[3u * i], pos[3u * i + 1u], pos[3u * i + 2u], 1.0f};
        float p[2];
        for (int r = 0; r < 2; r++) {
            p[r] = (MVP[4 * r] * x[0]) + (MVP[4 * r + 1] * x[1]) + (MVP[4 * r + 2] * x[2]) + (MVP[4 * r + 3] * x[3]);
            p[r] += 0.0f * vel[3u * i + (uint32_t)r];
        }
        const float phase = 1.000e-1f * pot[i];
        int32_t col[3];
        for (int c = 0; c < 3; c++) {
            const float sh = (float)(ORC_TAU * ((double)c / 3.0));
            col[c] = (int32_t)(100.0f * (0.5f * cosf((float)ORC_TAU * phase - sh) + 0.5f));
        }
        for (uint32_t smp = 0; smp < samples; smp++) {
            uint32_t h[4] = {0xB79ABC95u + smp, 0xE0DA3F84u + i, 0xAB75F07Bu + step, 0xCF52CA01u};
            orc_pcg4d(h);
            const float inv = (float)2.3283062977608182109179324470460414886474609375e-10;
            const float u2 = inv * (float)h[2], u3 = inv * (float)h[3];
            const float rad = sqrtf(-2.0f * logf(u2));
            const float o0 = 0.750f * (rad * cosf((float)ORC_TAU * u3));
            const float o1 = 0.750f * (rad * sinf((float)ORC_TAU * u3));
            const int cx = vis_to_int(o0 + -0.5f + half_y * p[0] + half_x);
            const int cy = vis_to_int(o1 + -0.5f + half_y * p[1] + half_y);
            if (0 <= cx && cx < (int)sizex && 0 <= cy && cy < (int)sizey) {
                int32_t* px = accum + 4u * ((size_t)sizex * (uint32_t)cy + (uint32_t)cx);
                for (int c = 0; c < 3; c++) {
#ifdef _OPENMP
#pragma omp atomic update
#endif
                    px[c] += col[c];
                }
#ifdef _OPENMP
#pragma omp atomic update
#endif
                px[3] += 1;
            }
        }
    }
    const double pscale = 0.01 / (double)samples * exp2(exposure);
    for (size_t k = 0; k < (size_t)sizex * sizey; k++) {
        for (int c = 0; c < 3; c++) {
            double v = pscale * (double)accum[4 * k + (size_t)c];
            if (tonemap) v = tanh(v);
            render[4 * k + (size_t)c] = (float)v;
        }
        render[4 * k + 3] = 1.0f;
    }
}

/* ---- initcond.c:11-255: initcond_generate ------------------------------- */
#define ORC_PI_4_3 4.18879020478639098461685784437267051226289253250014
#define ORC_PI_8_3 8.37758040957278196923371568874534102452578506500028
#define ORC_INV_PCG 2.3283062977608182109179324470460414886474609375e-10

static void orc_unit_direction(uint32_t a, uint32_t b, double* x, double* y, double* z) {
    const double r0 = ORC_INV_PCG * (double)a, r1 = ORC_INV_PCG * (double)b;
    const double phi = ORC_TAU * r0, the = acos(2.0 * r1 - 1.0);
    const double cp = cos(phi), sp = sin(phi), ct = cos(the), st = sin(the);
    *x = cp * st;
    *y = sp * st;
    *z = ct;
}

void orc_initcond(uint32_t n, double G, float* pos, float* vel, float* mas, float* rad) {
    const double radius = 1.000;
    const double volume = ORC_PI_4_3 * (radius * radius);
    const double body_mass = volume / (double)n;
    for (uint32_t i = 0; i < n; i++) {
        mas[i] = (float)body_mass;
        if (rad) rad[i] = 0.100f;
        uint32_t s[4] = {0xD88D5EFDu + i, 0x203F83D3u, 0x710BE493u, 0xA294E7F1u};
        orc_pcg4d(s);
        double p[3];
        orc_unit_direction(s[0], s[1], &p[0], &p[1], &p[2]);
        const double r2 = ORC_INV_PCG * (double)s[2];
        for (int k = 0; k < 3; k++) pos[3u * i + (uint32_t)k] = (float)(p[k] * (radius * cbrt(r2)));
    }
    for (uint32_t i = 0; i < n; i++) {
        const double p[3] = {pos[3u * i], pos[3u * i + 1u], pos[3u * i + 2u]};
        uint32_t s[4] = {0x4AFDC7CFu + i, 0xAE8D7CF2u, 0xE4827F00u, 0xE44CA389u};
        orc_pcg4d(s);
        double r[4];
        for (int k = 0; k < 4; k++) r[k] = ORC_INV_PCG * (double)s[k];
        double g[3] = {sqrt(-2.0 * log(r[0])) * cos(ORC_TAU * r[1]), sqrt(-2.0 * log(r[0])) * sin(ORC_TAU * r[1]),
                       sqrt(-2.0 * log(r[2])) * cos(ORC_TAU * r[3])};
        for (int k = 0; k < 3; k++) g[k] *= 1.000e-4;
        const double speed = sqrt((g[0] * g[0]) + (g[1] * g[1]) + (g[2] * g[2]));
        orc_pcg4d(s);
        double v[3];
        orc_unit_direction(s[0], s[1], &v[0], &v[1], &v[2]);
        for (int k = 0; k < 3; k++) {
            v[k] *= speed;
            v[k] += 4.000e-3 * sqrt(ORC_PI_8_3 * G) * p[k];
            vel[3u * i + (uint32_t)k] = (float)v[k];
        }
    }
}

/* ---- gravity.c:116-230 (compiled out by #if 0 in the reference) and
 * grid.c:197-536: the particle-mesh grid ----------------------------------- */
void orc_grid_deposit(uint32_t side, const float bmin[3], const float bmax[3], uint32_t n, const float* pos,
                      uint32_t step, uint32_t samples, int32_t* accum, float* poten) {
    const size_t cells = (size_t)side * side * side;
    const float wid[3] = {bmax[0] - bmin[0], bmax[1] - bmin[1], bmax[2] - bmin[2]};
    memset(accum, 0, sizeof(int32_t) * cells);
#pragma omp parallel for schedule(dynamic, 256)
    for (uint32_t i = 0; i < n; i++) {
        float pl[3];
        for (int k = 0; k < 3; k++) pl[k] = (pos[3u * i + (uint32_t)k] - bmin[k]) / wid[k];
        for (uint32_t j = 0; j < samples; j++) {
            uint32_t s[4] = {0xB79ABC95u + j, 0xE0DA3F84u + i, 0xAB75F07Bu + step, 0xCF52CA01u};
            orc_pcg4d(s);
            orc_pcg4d(s);
            float r[4];
            for (int k = 0; k < 4; k++) r[k] = (float)ORC_INV_PCG * (float)s[k];
            const float g[3] = {sqrtf(-2.0f * logf(r[0])) * cosf((float)ORC_TAU * r[1]),
                                sqrtf(-2.0f * logf(r[0])) * sinf((float)ORC_TAU * r[1]),
                                sqrtf(-2.0f * logf(r[2])) * cosf((float)ORC_TAU * r[3])};
            int c[3];
            for (int k = 0; k < 3; k++) c[k] = vis_to_int(0.500f * g[k] + (float)side * pl[k] + 0.5f);
            if (0 <= c[0] && c[0] < (int)side && 0 <= c[1] && c[1] < (int)side && 0 <= c[2] && c[2] < (int)side) {
                const size_t idx = (size_t)side * side * (uint32_t)c[2] + (size_t)side * (uint32_t)c[1] + (uint32_t)c[0];
#pragma omp atomic update
                accum[idx] += 1;
            }
        }
    }
    const double inv = 1.0 / (double)samples;
    for (size_t i = 0; i < cells; i++) poten[i] = (float)(inv * (double)accum[i]);
}

/* grid.c:281-315: the FP32 stencil -G / |x| at the cell corners. */
void orc_grid_stencil(uint32_t side, const float bmin[3], const float bmax[3], double G, float* out) {
    const float wid[3] = {bmax[0] - bmin[0], bmax[1] - bmin[1], bmax[2] - bmin[2]};
    for (uint32_t z = 0; z < side; z++)
        for (uint32_t y = 0; y < side; y++)
            for (uint32_t x = 0; x < side; x++) {
                const float p[3] = {wid[0] * ((float)x / (float)side) + bmin[0],
                                    wid[1] * ((float)y / (float)side) + bmin[1],
                                    wid[2] * ((float)z / (float)side) + bmin[2]};
                const float r2 = (p[0] * p[0]) + (p[1] * p[1]) + (p[2] * p[2]);
                const float inv = 0.0f < r2 ? 1.0f / sqrtf(r2) : 0.0f;
                out[(size_t)side * side * z + (size_t)side * y + x] = (float)(-G) * inv;
            }
}

/* In-place 1-D DFT of every line of a side^3 complex field along one axis
 * (stride 1, side or side^2), by the definition with an FP64 twiddle
 * table; sign -1 forward, +1 backward (unnormalised, as FFTW_BACKWARD). */
static void grid_dft_axis(uint32_t side, double* re, double* im, size_t stride, int sign) {
    const size_t cells = (size_t)side * side * side;
    double* wr = (double*)malloc(sizeof(double) * side);
    double* wi = (double*)malloc(sizeof(double) * side);
    for (uint32_t m = 0; m < side; m++) {
        wr[m] = cos(ORC_TAU * (double)m / (double)side);
        wi[m] = (double)sign * sin(ORC_TAU * (double)m / (double)side);
    }
    const size_t lines = cells / side;
#pragma omp parallel
    {
        double* tr = (double*)malloc(sizeof(double) * side);
        double* ti = (double*)malloc(sizeof(double) * side);
#pragma omp for schedule(static)
        for (size_t l = 0; l < lines; l++) {
            /* line l: the cells whose index has the axis digit zeroed */
            const size_t lo = l % stride, hi = l / stride;
            const size_t base = hi * stride * side + lo;
            for (uint32_t k = 0; k < side; k++) {
                double sr = 0.0, si = 0.0;
                uint32_t m = 0; /* j * k mod side */
                for (uint32_t j = 0; j < side; j++, m = (m + k >= side) ? m + k - side : m + k) {
                    const double xr = re[base + j * stride], xi = im[base + j * stride];
                    sr += xr * wr[m] - xi * wi[m];
                    si += xr * wi[m] + xi * wr[m];
                }
                tr[k] = sr;
                ti[k] = si;
            }
            for (uint32_t k = 0; k < side; k++) {
                re[base + k * stride] = tr[k];
                im[base + k * stride] = ti[k];
            }
        }
        free(tr);
        free(ti);
    }
    free(wr);
    free(wi);
}

static void grid_dft3(uint32_t side, double* re, double* im, int sign) {
    grid_dft_axis(side, re, im, 1, sign);
    grid_dft_axis(side, re, im, side, sign);
    grid_dft_axis(side, re, im, (size_t)side * side, sign);
}

void orc_grid_solve_fft(uint32_t side, const float bmin[3], const float bmax[3], double G, const float* samp,
                        double* out) {
    const size_t cells = (size_t)side * side * side;
    float* st = (float*)malloc(sizeof(float) * cells);
    double* sr = (double*)calloc(cells, sizeof(double));
    double* si = (double*)calloc(cells, sizeof(double));
    double* fr = (double*)calloc(cells, sizeof(double));
    double* fi = (double*)calloc(cells, sizeof(double));
    orc_grid_stencil(side, bmin, bmax, G, st);
    for (size_t i = 0; i < cells; i++) {
        sr[i] = st[i];
        fr[i] = samp[i];
    }
    grid_dft3(side, sr, si, -1);
    grid_dft3(side, fr, fi, -1);
    for (size_t i = 0; i < cells; i++) {
        const double a = fr[i], b = fi[i];
        fr[i] = a * sr[i] - b * si[i];
        fi[i] = a * si[i] + b * sr[i];
    }
    grid_dft3(side, fr, fi, +1);
    const uint32_t h = side / 2u;
    for (uint32_t z = 0; z < side; z++)
        for (uint32_t y = 0; y < side; y++)
            for (uint32_t x = 0; x < side; x++) {
                const size_t src = (size_t)side * side * ((z + h) % side) + (size_t)side * ((y + h) % side) +
                                   (x + h) % side;
                out[(size_t)side * side * z + (size_t)side * y + x] = fr[src];
            }
    free(st);
    free(sr);
    free(si);
    free(fr);
    free(fi);
}
