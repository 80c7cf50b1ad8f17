/*
 * fea_oracle_common.c -- integer half of the CPU restatement (test infrastructure
 * only; see fea_oracle.h): boundary detection, idx_map and the Eigen-compressed
 * sparsity pattern of the assembled matrices.
 */
#include "fea_oracle.h"

#include <stdlib.h>
#include <string.h>

static int cmp_u64(const void* a, const void* b) {
    uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
    return x < y ? -1 : (x > y ? 1 : 0);
}

/* Surface.cpp:104-122: edges[a][b]++ and edges[b][a]++ for every triangle edge,
 * then both ends of every (a, b) with count 1 are boundary points.  The count
 * of an undirected edge {a, b} (a != b) is the number of triangle edges joining
 * a and b; a degenerate edge a == b counts twice per use and is never 1. */
int64_t fo_boundary(int64_t V, int64_t T, const uint32_t* tri, uint8_t* on_boundary) {
    memset(on_boundary, 0, (size_t)V);
    uint64_t* keys = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)(3 * T + 1));
    int64_t n = 0;
    for (int64_t t = 0; t < T; t++) {
        for (int j = 0; j < 3; j++) {
            uint64_t a = tri[3 * t + j], b = tri[3 * t + (j + 1) % 3];
            if (a == b) continue;
            uint64_t lo = a < b ? a : b, hi = a < b ? b : a;
            keys[n++] = (lo << 32) | hi;
        }
    }
    qsort(keys, (size_t)n, sizeof(uint64_t), cmp_u64);
    for (int64_t i = 0; i < n;) {
        int64_t j = i;
        while (j < n && keys[j] == keys[i]) j++;
        if (j - i == 1) {
            on_boundary[keys[i] >> 32] = 1;
            on_boundary[keys[i] & 0xffffffffu] = 1;
        }
        i = j;
    }
    free(keys);
    int64_t nb = 0;
    for (int64_t v = 0; v < V; v++) nb += on_boundary[v] ? 1 : 0;
    return nb;
}

/* FEMContext.cpp:224-240: Dirichlet numbers the interior points in vertex
 * order (boundary -> -1); Neumann is the identity. */
int64_t fo_idx_map(int64_t V, const uint8_t* on_boundary, int bc, int32_t* idx_map) {
    int64_t idx = 0;
    for (int64_t i = 0; i < V; i++) {
        if (bc == 0) idx_map[i] = on_boundary[i] ? -1 : (int32_t)idx++;
        else idx_map[i] = (int32_t)idx++;
    }
    return idx;
}

typedef struct {
    int64_t N, nnz, T;
    int32_t* row_ptr;
    int32_t* col;
    int32_t* slot;
    int32_t* adv_slot;
} fo_pattern;

/* setFromTriplets (FEMContext.cpp:111,148): the triplet list is every (k, i, j)
 * that passes the BC filter of :99/:136, in loop order.  Restated semantics:
 * the matrix holds one entry per distinct (row, col), its value the sum of the
 * duplicates in triplet order; makeCompressed stores each outer vector with
 * sorted inner indices and keeps explicit zeros.  The stiffness and mass
 * filters are identical, so both matrices share this pattern; the symmetric
 * filter makes CSR and CSC index arrays coincide. */
void* fo_pattern_build(int64_t V, int64_t T, const uint32_t* tri, const uint8_t* on_b,
                       const int32_t* idx_map, int bc) {
    (void)V;
    fo_pattern* p = (fo_pattern*)calloc(1, sizeof(fo_pattern));
    int64_t N = 0;
    for (int64_t i = 0; i < V; i++)
        if (idx_map[i] >= 0 && idx_map[i] + 1 > N) N = idx_map[i] + 1;
    p->N = N;
    p->T = T;
    int64_t nt = 9 * T;
    p->slot = (int32_t*)malloc(sizeof(int32_t) * (size_t)(nt + 1));
    p->adv_slot = (int32_t*)malloc(sizeof(int32_t) * (size_t)(nt + 1));
    int64_t* cnt = (int64_t*)calloc((size_t)(N + 1), sizeof(int64_t));
    /* pass 1: triplets per row */
    for (int64_t k = 0; k < T; k++)
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                uint32_t vi = tri[3 * k + i], vj = tri[3 * k + j];
                int keep = (bc == 1) || (!on_b[vi] && !on_b[vj]);
                if (keep) cnt[idx_map[vi] + 1]++;
            }
    for (int64_t r = 0; r < N; r++) cnt[r + 1] += cnt[r];
    int64_t ntrip = cnt[N];
    /* pass 2: stable counting sort by row -> (col, triplet id) in triplet order */
    int32_t* bcol = (int32_t*)malloc(sizeof(int32_t) * (size_t)(ntrip + 1));
    int64_t* bid = (int64_t*)malloc(sizeof(int64_t) * (size_t)(ntrip + 1));
    int64_t* cur = (int64_t*)malloc(sizeof(int64_t) * (size_t)(N + 1));
    memcpy(cur, cnt, sizeof(int64_t) * (size_t)(N + 1));
    for (int64_t k = 0; k < T; k++)
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                int64_t id = 9 * k + 3 * i + j;
                uint32_t vi = tri[3 * k + i], vj = tri[3 * k + j];
                int keep = (bc == 1) || (!on_b[vi] && !on_b[vj]);
                p->slot[id] = -1;
                p->adv_slot[id] = -1;
                if (keep) {
                    int64_t pos = cur[idx_map[vi]]++;
                    bcol[pos] = idx_map[vj];
                    bid[pos] = id;
                }
            }
    /* pass 3: per row, stable insertion sort by column, then collapse */
    p->row_ptr = (int32_t*)malloc(sizeof(int32_t) * (size_t)(N + 1));
    p->col = (int32_t*)malloc(sizeof(int32_t) * (size_t)(ntrip + 1));
    int64_t nnz = 0;
    for (int64_t r = 0; r < N; r++) {
        int64_t s = cnt[r], e = cnt[r + 1];
        for (int64_t a = s + 1; a < e; a++) {
            int32_t c = bcol[a];
            int64_t d = bid[a];
            int64_t b = a - 1;
            while (b >= s && bcol[b] > c) {
                bcol[b + 1] = bcol[b];
                bid[b + 1] = bid[b];
                b--;
            }
            bcol[b + 1] = c;
            bid[b + 1] = d;
        }
        p->row_ptr[r] = (int32_t)nnz;
        for (int64_t a = s; a < e; a++) {
            if (a == s || bcol[a] != bcol[a - 1]) p->col[nnz++] = bcol[a];
            p->slot[bid[a]] = (int32_t)(nnz - 1);
        }
    }
    p->row_ptr[N] = (int32_t)nnz;
    p->nnz = nnz;
    /* advection filter (FEMContext.cpp:188) ignores the BC: only entries whose
     * two vertices are both off the boundary */
    for (int64_t k = 0; k < T; k++)
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                int64_t id = 9 * k + 3 * i + j;
                uint32_t vi = tri[3 * k + i], vj = tri[3 * k + j];
                if (!on_b[vi] && !on_b[vj]) p->adv_slot[id] = p->slot[id];
            }
    free(bcol);
    free(bid);
    free(cur);
    free(cnt);
    return p;
}

int64_t fo_pattern_nnz(const void* h) { return ((const fo_pattern*)h)->nnz; }
int64_t fo_pattern_rows(const void* h) { return ((const fo_pattern*)h)->N; }

void fo_pattern_copy(const void* h, int32_t* row_ptr, int32_t* col, int32_t* slot, int32_t* adv_slot) {
    const fo_pattern* p = (const fo_pattern*)h;
    if (row_ptr) memcpy(row_ptr, p->row_ptr, sizeof(int32_t) * (size_t)(p->N + 1));
    if (col) memcpy(col, p->col, sizeof(int32_t) * (size_t)p->nnz);
    if (slot) memcpy(slot, p->slot, sizeof(int32_t) * (size_t)(9 * p->T));
    if (adv_slot) memcpy(adv_slot, p->adv_slot, sizeof(int32_t) * (size_t)(9 * p->T));
}

void fo_pattern_free(void* h) {
    fo_pattern* p = (fo_pattern*)h;
    if (!p) return;
    free(p->row_ptr);
    free(p->col);
    free(p->slot);
    free(p->adv_slot);
    free(p);
}
