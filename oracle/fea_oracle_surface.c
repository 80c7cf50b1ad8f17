/*
 * fea_oracle_surface.c -- the steps after the solve in the application's
 * frame (test infrastructure only; see fea_oracle.h).
 *
 *   - extruded smooth normals        shaders/FEM/smooth_normals.glsl:30-57
 *                                    (Surface::calculate_normals, Surface.cpp:287-306)
 *   - iso-clipped .ply geometry      Surface::export_to_ply, Surface.cpp:138-285
 *
 * Float arithmetic in the reference's operation order, without contraction
 * (built with -ffp-contract=off).  glm::mix(x, y, a) is x * (1 - a) + y * a.
 * The shader accumulates with float atomics in no fixed order; here the sum
 * runs in triangle order.
 */
#include <stdlib.h>
#include <string.h>

#include "fea_oracle.h"

static void sub3(const float* a, const float* b, float* o) {
    o[0] = a[0] - b[0];
    o[1] = a[1] - b[1];
    o[2] = a[2] - b[2];
}

void fo_smooth_normals_f32(int64_t V, int64_t T, const float* xyz, const uint32_t* tri, const float* normals,
                           const float* values, float extrusion, float* out) {
    memset(out, 0, sizeof(float) * 3 * (size_t)V);
    for (int64_t k = 0; k < T; k++) {
        float p[3][3];
        for (int i = 0; i < 3; i++) {
            const uint32_t v = tri[3 * k + i];
            float s = values[v] > 0.0f ? values[v] : 0.0f;
            s = extrusion * s;
            if (s > 1.0f) s = 1.0f;
            for (int d = 0; d < 3; d++) p[i][d] = xyz[3 * v + d] + s * normals[3 * v + d];
        }
        float e1[3], e2[3], n[3];
        sub3(p[1], p[0], e1);
        sub3(p[2], p[0], e2);
        n[0] = e1[1] * e2[2] - e1[2] * e2[1];
        n[1] = e1[2] * e2[0] - e1[0] * e2[2];
        n[2] = e1[0] * e2[1] - e1[1] * e2[0];
        for (int i = 0; i < 3; i++)
            for (int d = 0; d < 3; d++) out[3 * tri[3 * k + i] + d] += n[d];
    }
}

/* ---- iso-clipped export ----------------------------------------------------- */

typedef struct {
    uint32_t key[3];
    int64_t idx;
} fo_slot;

typedef struct {
    fo_slot* tab;
    int64_t cap;
    float* pos;
    float* val;
    int64_t n, cap_v;
} fo_dedup;

static uint32_t bits_of(float f) {
    uint32_t u;
    if (f == 0.0f) f = 0.0f; /* -0 and +0 compare equal */
    memcpy(&u, &f, 4);
    return u;
}

static uint64_t hash3(const uint32_t* k) {
    uint64_t h = 1469598103934665603ull;
    for (int i = 0; i < 3; i++) h = (h ^ k[i]) * 1099511628211ull;
    return h;
}

/* clipped_position_map: the index of the first position equal to p */
static int64_t dedup_add(fo_dedup* D, const float* p, float value) {
    uint32_t k[3] = {bits_of(p[0]), bits_of(p[1]), bits_of(p[2])};
    int64_t h = (int64_t)(hash3(k) & (uint64_t)(D->cap - 1));
    for (;;) {
        fo_slot* s = &D->tab[h];
        if (s->idx < 0) {
            if (D->n >= D->cap_v) return -1;
            memcpy(s->key, k, sizeof(k));
            s->idx = D->n;
            memcpy(D->pos + 3 * D->n, p, 3 * sizeof(float));
            D->val[D->n] = value;
            return D->n++;
        }
        if (!memcmp(s->key, k, sizeof(k))) return s->idx;
        h = (h + 1) & (D->cap - 1);
    }
}

static void extruded(const float* xyz, const float* nrm, const float* values, float e, uint32_t v, float* o) {
    const float s = values[v] * (e > 0.0f ? e : 0.0f);
    for (int d = 0; d < 3; d++) o[d] = s * nrm[3 * v + d] + xyz[3 * v + d];
}

static void along(const float* xyz, const float* nrm, float scale, uint32_t v, float* o) {
    for (int d = 0; d < 3; d++) o[d] = scale * nrm[3 * v + d] + xyz[3 * v + d];
}

static void mix3(const float* x, const float* y, float a, float* o) {
    for (int d = 0; d < 3; d++) o[d] = x[d] * (1.0f - a) + y[d] * a;
}

int64_t fo_ply_clip(int64_t V, int64_t T, const float* xyz, const uint32_t* tri, const float* nrm,
                    const float* values, float e, float threshold, int mesh_type, float* pos_out,
                    float* val_out, int64_t cap_v, uint32_t* tri_out, int64_t cap_t, int64_t* ntri) {
    (void)V;
    fo_dedup D;
    D.cap = 1;
    while (D.cap < 2 * cap_v + 2) D.cap <<= 1;
    D.tab = (fo_slot*)malloc(sizeof(fo_slot) * (size_t)D.cap);
    for (int64_t i = 0; i < D.cap; i++) D.tab[i].idx = -1;
    D.pos = pos_out;
    D.val = val_out;
    D.n = 0;
    D.cap_v = cap_v;
    int64_t nt = 0;
#define EMIT(a, b, c)                                  \
    do {                                               \
        if (nt < cap_t) {                              \
            tri_out[3 * nt + 0] = (uint32_t)(a);       \
            tri_out[3 * nt + 1] = (uint32_t)(b);       \
            tri_out[3 * nt + 2] = (uint32_t)(c);       \
        }                                              \
        nt++;                                          \
    } while (0)
    for (int64_t k = 0; k < T; k++) {
        const uint32_t t[3] = {tri[3 * k], tri[3 * k + 1], tri[3 * k + 2]};
        int above[3], count = 0;
        for (int i = 0; i < 3; i++) {
            above[i] = (double)(values[t[i]] - threshold) >= 1e-9;
            count += above[i];
        }
        if (count == 1) {
            const int ai = above[0] ? 0 : above[1] ? 1 : 2;
            int64_t ct[3];
            float ea[3];
            extruded(xyz, nrm, values, e, t[ai], ea);
            for (int i = 0; i < 3; i++) {
                float p[3];
                float value;
                if (i != ai) {
                    float ei[3];
                    extruded(xyz, nrm, values, e, t[i], ei);
                    const float a = (threshold - values[t[i]]) / (values[t[ai]] - values[t[i]]);
                    mix3(ei, ea, a, p);
                    value = threshold;
                } else {
                    memcpy(p, ea, sizeof(p));
                    value = values[t[ai]];
                }
                ct[i] = dedup_add(&D, p, value);
            }
            EMIT(ct[0], ct[1], ct[2]);
            if (mesh_type != 0) {
                int64_t pr[3];
                for (int i = 0; i < 3; i++) {
                    if (i != ai) {
                        pr[i] = ct[i];
                    } else {
                        const float sc = mesh_type == 2 ? threshold - values[t[i]] * e : threshold * e;
                        float p[3];
                        along(xyz, nrm, sc, t[i], p);
                        pr[i] = dedup_add(&D, p, threshold);
                    }
                }
                EMIT(pr[0], pr[1], pr[2]);
            }
        } else if (count == 2) {
            const int a1 = above[0] ? 0 : 1;
            const int a2 = above[0] && above[1] ? 1 : 2;
            const int bi = 3 - (a1 + a2);
            float pa1[3], pa2[3], pb[3], m1[3], m2[3];
            extruded(xyz, nrm, values, e, t[a1], pa1);
            extruded(xyz, nrm, values, e, t[a2], pa2);
            extruded(xyz, nrm, values, e, t[bi], pb);
            mix3(pb, pa1, (threshold - values[t[bi]]) / (values[t[a1]] - values[t[bi]]), m1);
            mix3(pb, pa2, (threshold - values[t[bi]]) / (values[t[a2]] - values[t[bi]]), m2);
            const int64_t ia1 = dedup_add(&D, pa1, values[t[a1]]);
            const int64_t ia2 = dedup_add(&D, pa2, values[t[a2]]);
            const int64_t ib1 = dedup_add(&D, m1, threshold);
            const int64_t ib2 = dedup_add(&D, m2, threshold);
            EMIT(ib1, ia1, ib2);
            EMIT(ib2, ia1, ia2);
            if (mesh_type != 0) {
                float q1[3], q2[3];
                if (mesh_type == 2) {
                    along(xyz, nrm, threshold - values[t[a1]] * e, t[a1], q1);
                    along(xyz, nrm, threshold - values[t[a2]] * e, t[a2], q2);
                } else {
                    along(xyz, nrm, threshold * e, t[a1], q1);
                    along(xyz, nrm, threshold * e, t[a2], q2);
                }
                const int64_t iq1 = dedup_add(&D, q1, values[t[a1]]);
                const int64_t iq2 = dedup_add(&D, q2, values[t[a2]]);
                EMIT(ib1, iq1, ib2);
                EMIT(ib2, iq1, iq2);
            }
        } else if (count == 3) {
            int64_t ct[3];
            for (int i = 0; i < 3; i++) {
                float p[3];
                extruded(xyz, nrm, values, e, t[i], p);
                ct[i] = dedup_add(&D, p, values[t[i]]);
            }
            EMIT(ct[0], ct[1], ct[2]);
            if (mesh_type != 0) {
                int64_t pr[3];
                for (int i = 0; i < 3; i++) {
                    const float sc = mesh_type == 2 ? threshold - values[t[i]] * e : threshold * e;
                    float p[3];
                    along(xyz, nrm, sc, t[i], p);
                    pr[i] = dedup_add(&D, p, threshold);
                }
                EMIT(pr[0], pr[1], pr[2]);
            }
        }
    }
#undef EMIT
    free(D.tab);
    *ntri = nt;
    return D.n;
}
