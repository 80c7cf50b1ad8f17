// surface.cu -- the steps after the solve in the application's frame:
// extruded smooth normals and the clipping stage of the .ply export.
//
// Smooth normals (shaders/FEM/smooth_normals.glsl:30-57, dispatched by
// Surface::calculate_normals, Surface.cpp:287-306): every triangle's corners
// move along their normals by min(1, e * max(0, value)); the cross product of
// the moved triangle's edges is added to its three vertices.  The shader adds
// with float atomics in no fixed order; here one kernel writes each face
// normal and a second sums, per vertex, the normals of its triangles in
// ascending triangle order (a vertex -> triangle list built once per mesh),
// so the result is the same on every run.
//
// Export clipping (Surface::export_to_ply, Surface.cpp:138-285): per triangle
// the positions the reference adds to its position map (up to 6, in the same
// order) and the triangles it emits (up to 4, as references to those slots).
// Float arithmetic is rounded at every operation (no contraction), so the
// positions equal the reference's bit for bit and the host's first-seen
// deduplication numbers them the same way.
#include "fea_internal.cuh"

namespace fea {
namespace {

__device__ __forceinline__ float clampe(float v, float e) {  // min(1, e * max(0, v))
    const float s = __fmul_rn(e, fmaxf(0.0f, v));
    return fminf(1.0f, s);
}

__global__ void k_face_normals(int64_t T, const float* __restrict__ xyz, const uint32_t* __restrict__ tri,
                               const float* __restrict__ nrm, const float* __restrict__ val, float e, float* face) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < T; k += (int64_t)gridDim.x * blockDim.x) {
        float p[3][3];
#pragma unroll
        for (int i = 0; i < 3; i++) {
            const uint32_t v = tri[3 * k + i];
            const float s = clampe(val[v], e);
#pragma unroll
            for (int d = 0; d < 3; d++) p[i][d] = __fadd_rn(xyz[3 * v + d], __fmul_rn(s, nrm[3 * v + d]));
        }
        float a[3], b[3];
#pragma unroll
        for (int d = 0; d < 3; d++) {
            a[d] = __fsub_rn(p[1][d], p[0][d]);
            b[d] = __fsub_rn(p[2][d], p[0][d]);
        }
        face[3 * k + 0] = __fsub_rn(__fmul_rn(a[1], b[2]), __fmul_rn(a[2], b[1]));
        face[3 * k + 1] = __fsub_rn(__fmul_rn(a[2], b[0]), __fmul_rn(a[0], b[2]));
        face[3 * k + 2] = __fsub_rn(__fmul_rn(a[0], b[1]), __fmul_rn(a[1], b[0]));
    }
}

__global__ void k_vertex_normals(int64_t V, const int32_t* __restrict__ vt_ptr, const int32_t* __restrict__ vt_tri,
                                 const float* __restrict__ face, float* out) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < V; v += (int64_t)gridDim.x * blockDim.x) {
        float s[3] = {0.f, 0.f, 0.f};
        for (int32_t j = vt_ptr[v]; j < vt_ptr[v + 1]; j++) {
            const int32_t k = vt_tri[j];
#pragma unroll
            for (int d = 0; d < 3; d++) s[d] = __fadd_rn(s[d], face[3 * (int64_t)k + d]);
        }
#pragma unroll
        for (int d = 0; d < 3; d++) out[3 * v + d] = s[d];
    }
}

// vertex -> incident triangles: counts, then slots, then each list sorted by
// triangle number (the fill order of the atomics is arbitrary)
__global__ void k_vt_count(int64_t T, const uint32_t* __restrict__ tri, int32_t* cnt) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < 3 * T; k += (int64_t)gridDim.x * blockDim.x)
        atomicAdd(&cnt[tri[k]], 1);
}

__global__ void k_vt_fill(int64_t T, const uint32_t* __restrict__ tri, const int32_t* __restrict__ ptr, int32_t* cur,
                          int32_t* vt_tri) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < 3 * T; k += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t v = tri[k];
        const int32_t at = atomicAdd(&cur[v], 1);
        vt_tri[ptr[v] + at] = (int32_t)(k / 3);
    }
}

__global__ void k_vt_sort(int64_t V, const int32_t* __restrict__ ptr, int32_t* vt_tri) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < V; v += (int64_t)gridDim.x * blockDim.x) {
        const int32_t b = ptr[v], e = ptr[v + 1];
        for (int32_t i = b + 1; i < e; i++) {
            const int32_t x = vt_tri[i];
            int32_t j = i - 1;
            while (j >= b && vt_tri[j] > x) {
                vt_tri[j + 1] = vt_tri[j];
                j--;
            }
            vt_tri[j + 1] = x;
        }
    }
}

// ---- export clipping ------------------------------------------------------------

struct ClipIn {
    const float* xyz;
    const float* nrm;
    const float* val;
    float e, thr;
};

// values[v] * max(0, e) * n + p
__device__ __forceinline__ void extruded(const ClipIn& c, uint32_t v, float* o) {
    const float s = __fmul_rn(c.val[v], fmaxf(0.0f, c.e));
#pragma unroll
    for (int d = 0; d < 3; d++) o[d] = __fadd_rn(__fmul_rn(s, c.nrm[3 * v + d]), c.xyz[3 * v + d]);
}

__device__ __forceinline__ void along(const ClipIn& c, float scale, uint32_t v, float* o) {
#pragma unroll
    for (int d = 0; d < 3; d++) o[d] = __fadd_rn(__fmul_rn(scale, c.nrm[3 * v + d]), c.xyz[3 * v + d]);
}

// glm::mix(x, y, a) = x * (1 - a) + y * a
__device__ __forceinline__ void mix3(const float* x, const float* y, float a, float* o) {
    const float b = __fsub_rn(1.0f, a);
#pragma unroll
    for (int d = 0; d < 3; d++) o[d] = __fadd_rn(__fmul_rn(x[d], b), __fmul_rn(y[d], a));
}

// Per triangle k: slots 6k..6k+5 (position, value, used) and triangles
// 4k..4k+3 (three slot numbers, or -1 when not emitted), in the reference's
// order of add_clipped_position calls and emitted triangles.
__global__ void k_ply_clip(int64_t T, const uint32_t* __restrict__ tri, ClipIn c, int mesh_type, float* pos,
                           float* pval, uint8_t* used, int32_t* otri) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < T; k += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t t[3] = {tri[3 * k], tri[3 * k + 1], tri[3 * k + 2]};
        const int64_t s0 = 6 * k;
#pragma unroll
        for (int j = 0; j < 6; j++) used[s0 + j] = 0;
#pragma unroll
        for (int j = 0; j < 12; j++) otri[12 * k + j] = -1;
        auto put = [&](int j, const float* p, float v) {
#pragma unroll
            for (int d = 0; d < 3; d++) pos[3 * (s0 + j) + d] = p[d];
            pval[s0 + j] = v;
            used[s0 + j] = 1;
        };
        auto emit = [&](int q, int a, int b, int cc) {
            otri[12 * k + 3 * q + 0] = (int32_t)(s0 + a);
            otri[12 * k + 3 * q + 1] = (int32_t)(s0 + b);
            otri[12 * k + 3 * q + 2] = (int32_t)(s0 + cc);
        };
        int above[3], count = 0;
#pragma unroll
        for (int i = 0; i < 3; i++) {
            above[i] = (double)__fsub_rn(c.val[t[i]], c.thr) >= 1e-9;
            count += above[i];
        }
        const float thr = c.thr, e = c.e;
        if (count == 1) {
            const int ai = above[0] ? 0 : above[1] ? 1 : 2;
            float ea[3];
            extruded(c, t[ai], ea);
            for (int i = 0; i < 3; i++) {
                float p[3];
                if (i != ai) {
                    float ei[3];
                    extruded(c, t[i], ei);
                    const float a = __fdiv_rn(__fsub_rn(thr, c.val[t[i]]), __fsub_rn(c.val[t[ai]], c.val[t[i]]));
                    mix3(ei, ea, a, p);
                    put(i, p, thr);
                } else {
                    put(i, ea, c.val[t[ai]]);
                }
            }
            emit(0, 0, 1, 2);
            if (mesh_type != 0) {
                const float sc = mesh_type == 2 ? __fsub_rn(thr, __fmul_rn(c.val[t[ai]], e)) : __fmul_rn(thr, e);
                float p[3];
                along(c, sc, t[ai], p);
                put(3, p, thr);
                int pr[3] = {0, 1, 2};
                pr[ai] = 3;
                emit(1, pr[0], pr[1], pr[2]);
            }
        } else if (count == 2) {
            const int a1 = above[0] ? 0 : 1;
            const int a2 = above[0] && above[1] ? 1 : 2;
            const int bi = 3 - (a1 + a2);
            float pa1[3], pa2[3], pb[3], m1[3], m2[3];
            extruded(c, t[a1], pa1);
            extruded(c, t[a2], pa2);
            extruded(c, t[bi], pb);
            mix3(pb, pa1, __fdiv_rn(__fsub_rn(thr, c.val[t[bi]]), __fsub_rn(c.val[t[a1]], c.val[t[bi]])), m1);
            mix3(pb, pa2, __fdiv_rn(__fsub_rn(thr, c.val[t[bi]]), __fsub_rn(c.val[t[a2]], c.val[t[bi]])), m2);
            put(0, pa1, c.val[t[a1]]);
            put(1, pa2, c.val[t[a2]]);
            put(2, m1, thr);
            put(3, m2, thr);
            emit(0, 2, 0, 3);
            emit(1, 3, 0, 1);
            if (mesh_type != 0) {
                float q1[3], q2[3];
                if (mesh_type == 2) {
                    along(c, __fsub_rn(thr, __fmul_rn(c.val[t[a1]], e)), t[a1], q1);
                    along(c, __fsub_rn(thr, __fmul_rn(c.val[t[a2]], e)), t[a2], q2);
                } else {
                    along(c, __fmul_rn(thr, e), t[a1], q1);
                    along(c, __fmul_rn(thr, e), t[a2], q2);
                }
                put(4, q1, c.val[t[a1]]);
                put(5, q2, c.val[t[a2]]);
                emit(2, 2, 4, 3);
                emit(3, 3, 4, 5);
            }
        } else if (count == 3) {
            for (int i = 0; i < 3; i++) {
                float p[3];
                extruded(c, t[i], p);
                put(i, p, c.val[t[i]]);
            }
            emit(0, 0, 1, 2);
            if (mesh_type != 0) {
                for (int i = 0; i < 3; i++) {
                    const float sc = mesh_type == 2 ? __fsub_rn(thr, __fmul_rn(c.val[t[i]], e)) : __fmul_rn(thr, e);
                    float p[3];
                    along(c, sc, t[i], p);
                    put(3 + i, p, thr);
                }
                emit(1, 3, 4, 5);
            }
        }
    }
}

}  // namespace

void build_vertex_triangles(const uint32_t* tri, int64_t T, int64_t V, int32_t* vt_ptr, int32_t* vt_tri,
                            cudaStream_t st) {
    DeviceArena tmp;
    int32_t* cnt = tmp.alloc<int32_t>(V + 1);
    FEA_CUDA_TRY(cudaMemsetAsync(cnt, 0, sizeof(int32_t) * (V + 1), st));
    k_vt_count<<<launch_grid(3 * T), kBlock, 0, st>>>(T, tri, cnt);
    FEA_CHECK_LAUNCH();
    exclusive_scan_i32(cnt, vt_ptr, V, st);
    FEA_CUDA_TRY(cudaMemsetAsync(cnt, 0, sizeof(int32_t) * (V + 1), st));
    k_vt_fill<<<launch_grid(3 * T), kBlock, 0, st>>>(T, tri, vt_ptr, cnt, vt_tri);
    FEA_CHECK_LAUNCH();
    k_vt_sort<<<launch_grid(V), kBlock, 0, st>>>(V, vt_ptr, vt_tri);
    FEA_CHECK_LAUNCH();
    FEA_CUDA_TRY(cudaStreamSynchronize(st));
}

void smooth_normals(const float* xyz, const uint32_t* tri, int64_t T, int64_t V, const int32_t* vt_ptr,
                    const int32_t* vt_tri, const float* nrm, const float* val, float e, float* face, float* out,
                    cudaStream_t st) {
    if (T > 0) {
        k_face_normals<<<launch_grid(T), kBlock, 0, st>>>(T, xyz, tri, nrm, val, e, face);
        FEA_CHECK_LAUNCH();
    }
    k_vertex_normals<<<launch_grid(V), kBlock, 0, st>>>(V, vt_ptr, vt_tri, face, out);
    FEA_CHECK_LAUNCH();
}

void ply_clip(const float* xyz, const uint32_t* tri, int64_t T, const float* nrm, const float* val, float e,
              float threshold, int mesh_type, float* pos, float* pval, uint8_t* used, int32_t* otri,
              cudaStream_t st) {
    if (T == 0) return;
    k_ply_clip<<<launch_grid(T), kBlock, 0, st>>>(T, tri, ClipIn{xyz, nrm, val, e, threshold}, mesh_type, pos, pval,
                                                  used, otri);
    FEA_CHECK_LAUNCH();
}

}  // namespace fea
