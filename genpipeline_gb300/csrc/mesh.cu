// mesh.cu -- isosurface of a density grid on the device, for the STL export that follows a
// SIMP run (density_to_stl, topology/mesh_export.py:7-67; the reference extracts it on the
// host with skimage's marching cubes).
//
// Marching cubes over the (nx-1)(ny-1)(nz-1) cells between voxel centres. The case table is
// generated here, not copied: for each of the 256 inside/outside patterns of a cell's
// corners (inside = value >= level), every face contributes the segments that join its cut
// edges; a face with all four edges cut (diagonal corners inside) separates its two inside
// corners, a rule that depends on the face alone, so the two cells sharing a face agree and
// the surface has no cracks. The segments close into loops; each loop is oriented so that its
// normal points from the inside corners to the outside ones (the density's descent
// direction). A loop of three is one triangle; a longer loop is fanned around the mean of its
// vertices, so that every edge between two loop vertices is a face segment, shared with the
// neighbouring cell (a fan between loop vertices can lay a diagonal flat on an ambiguous face,
// where it overlaps the neighbour's). Vertices lie on the cut edges at the linear
// interpolation of the level, computed from the lower-indexed end of each edge so that the
// cells sharing an edge produce bit-identical points.
//
// Corner c of cell (i, j, k) is (i + cx, j + cy, k + cz) with (cx, cy, cz) the FEM corner order
// (0,0,0),(1,0,0),(1,1,0),(0,1,0),(0,0,1),(1,0,1),(1,1,1),(0,1,1). Triangles are written in
// cell order (C order of (i, j, k)), then in table order, as 9 floats (three vertices, scaled
// by the voxel size).
#include <math.h>
#include <string.h>

#include <utility>
#include <vector>

#include "internal.h"

namespace gbs {

constexpr int kMcMaxTri = 12;

struct McTable {
    unsigned char ntri[256];     // triangles of the case
    unsigned char nloop[256];    // loops of the case (at most 4)
    unsigned char len[256][4];   // edges per loop
    signed char edge[256][12];   // the loops' edges, one after the other
};

static const int kMcCorner[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
static const int kMcEdge[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6},
                                   {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};
// faces as corner cycles
static const int kMcFace[6][4] = {{0, 1, 2, 3}, {4, 5, 6, 7}, {0, 1, 5, 4}, {3, 2, 6, 7}, {0, 3, 7, 4}, {1, 2, 6, 5}};

static int mc_edge_of(int a, int b) {
    for (int e = 0; e < 12; ++e)
        if ((kMcEdge[e][0] == a && kMcEdge[e][1] == b) || (kMcEdge[e][0] == b && kMcEdge[e][1] == a)) return e;
    return -1;
}

static McTable mc_build_table() {
    McTable T;
    memset(&T, 0, sizeof T);
    for (int cs = 0; cs < 256; ++cs) {
        auto in = [&](int c) { return (cs >> c) & 1; };
        // neighbours of each cut edge along the face segments
        int nb[12][2];
        int deg[12] = {0};
        for (int e = 0; e < 12; ++e) nb[e][0] = nb[e][1] = -1;
        auto link = [&](int e0, int e1) {
            nb[e0][deg[e0]++] = e1;
            nb[e1][deg[e1]++] = e0;
        };
        for (int f = 0; f < 6; ++f) {
            const int *q = kMcFace[f];
            int cut[4], nc = 0;
            for (int s = 0; s < 4; ++s)
                if (in(q[s]) != in(q[(s + 1) % 4])) cut[nc++] = s;  // side s joins q[s], q[s+1]
            if (nc == 2) {
                link(mc_edge_of(q[cut[0]], q[(cut[0] + 1) % 4]), mc_edge_of(q[cut[1]], q[(cut[1] + 1) % 4]));
            } else if (nc == 4) {
                // inside corners are q[0], q[2] or q[1], q[3]: cut each inside corner off
                for (int s = 0; s < 4; ++s)
                    if (in(q[s])) {
                        const int prev = (s + 3) % 4;
                        link(mc_edge_of(q[prev], q[s]), mc_edge_of(q[s], q[(s + 1) % 4]));
                    }
            }
        }
        bool used[12] = {false};
        int nt = 0, nl = 0, ne = 0;
        for (int e0 = 0; e0 < 12; ++e0) {
            if (deg[e0] == 0 || used[e0]) continue;
            std::vector<int> loop;
            int prev = -1, cur = e0;
            while (true) {
                loop.push_back(cur);
                used[cur] = true;
                const int nx = nb[cur][0] != prev ? nb[cur][0] : nb[cur][1];
                prev = cur;
                cur = nx;
                if (cur == e0 || cur < 0) break;
            }
            // orientation: Newell normal of the edge midpoints against inside -> outside
            double mid[12][3];
            for (size_t t = 0; t < loop.size(); ++t)
                for (int d = 0; d < 3; ++d)
                    mid[t][d] = 0.5 * (kMcCorner[kMcEdge[loop[t]][0]][d] + kMcCorner[kMcEdge[loop[t]][1]][d]);
            double nrm[3] = {0, 0, 0}, dir[3] = {0, 0, 0};
            for (size_t t = 0; t < loop.size(); ++t) {
                const double *p = mid[t], *q = mid[(t + 1) % loop.size()];
                nrm[0] += (p[1] - q[1]) * (p[2] + q[2]);
                nrm[1] += (p[2] - q[2]) * (p[0] + q[0]);
                nrm[2] += (p[0] - q[0]) * (p[1] + q[1]);
                const int a = kMcEdge[loop[t]][0], b = kMcEdge[loop[t]][1];
                const int ci = in(a) ? a : b, co = in(a) ? b : a;
                for (int d = 0; d < 3; ++d) dir[d] += kMcCorner[co][d] - kMcCorner[ci][d];
            }
            if (nrm[0] * dir[0] + nrm[1] * dir[1] + nrm[2] * dir[2] < 0) {
                for (size_t t = 1, u = loop.size() - 1; t < u; ++t, --u) std::swap(loop[t], loop[u]);
            }
            T.len[cs][nl++] = (unsigned char)loop.size();  // every cut edge is on one loop: ne <= 12
            for (int e : loop) T.edge[cs][ne++] = (signed char)e;
            nt += loop.size() == 3 ? 1 : (int)loop.size();
        }
        T.ntri[cs] = (unsigned char)nt;
        T.nloop[cs] = (unsigned char)nl;
    }
    return T;
}

static const McTable &mc_table() {
    static const McTable T = mc_build_table();
    return T;
}

__device__ __forceinline__ int mc_case(const float *__restrict__ v, int i, int j, int k, int ny, int nz, float level,
                                       float (&c)[8]) {
    int cs = 0;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const int cx = (q == 1 || q == 2 || q == 5 || q == 6), cy = (q == 2 || q == 3 || q == 6 || q == 7), cz = q >= 4;
        c[q] = v[((long long)(i + cx) * ny + (j + cy)) * nz + (k + cz)];
        cs |= (c[q] >= level) << q;
    }
    return cs;
}

constexpr int kMcBlock = 256;

// Triangles per block of cells.
__global__ void mc_count_kernel(const float *__restrict__ v, int nx, int ny, int nz, float level, const McTable T,
                                long long *block_tris) {
    const long long ncell = (long long)(nx - 1) * (ny - 1) * (nz - 1);
    const long long id = blockIdx.x * (long long)kMcBlock + threadIdx.x;
    int n = 0;
    if (id < ncell) {
        const int k = (int)(id % (nz - 1)), j = (int)((id / (nz - 1)) % (ny - 1)), i = (int)(id / ((long long)(nz - 1) * (ny - 1)));
        float c[8];
        n = T.ntri[mc_case(v, i, j, k, ny, nz, level, c)];
    }
    __shared__ int ws[kMcBlock / 32];
    int s = n;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        long long t = 0;
        for (int w = 0; w < kMcBlock / 32; ++w) t += ws[w];
        block_tris[blockIdx.x] = t;
    }
}

// Exclusive scan of the block totals (one block, in chunks); total in block_tris[nb].
__global__ void mc_scan_kernel(long long *block_tris, long long nb) {
    __shared__ long long buf[1024];
    __shared__ long long carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (long long base = 0; base < nb; base += 1024) {
        const long long id = base + threadIdx.x;
        const long long x = id < nb ? block_tris[id] : 0;
        buf[threadIdx.x] = x;
        __syncthreads();
        for (int o = 1; o < 1024; o <<= 1) {  // Hillis-Steele inclusive scan
            const long long y = threadIdx.x >= o ? buf[threadIdx.x - o] : 0;
            __syncthreads();
            buf[threadIdx.x] += y;
            __syncthreads();
        }
        if (id < nb) block_tris[id] = carry + buf[threadIdx.x] - x;
        __syncthreads();
        if (threadIdx.x == 1023) carry += buf[1023];
        __syncthreads();
    }
    if (threadIdx.x == 0) block_tris[nb] = carry;
}

__device__ __forceinline__ void mc_vertex(int e, int i, int j, int k, const float (&c)[8], float level, float sx,
                                          float sy, float sz, float *out) {
    const int ea[12] = {0, 1, 2, 3, 4, 5, 6, 7, 0, 1, 2, 3}, eb[12] = {1, 2, 3, 0, 5, 6, 7, 4, 4, 5, 6, 7};
    int a = ea[e], b = eb[e];
    const int ax = (a == 1 || a == 2 || a == 5 || a == 6), ay = (a == 2 || a == 3 || a == 6 || a == 7), az = a >= 4;
    const int bx = (b == 1 || b == 2 || b == 5 || b == 6), by = (b == 2 || b == 3 || b == 6 || b == 7), bz = b >= 4;
    // interpolate from the lower grid point of the edge (shared edges give identical points)
    const bool swap = ax + ay + az > bx + by + bz;
    const float va = swap ? c[b] : c[a], vb = swap ? c[a] : c[b];
    const float t = (level - va) / (vb - va);
    const float px = (float)(i + (swap ? bx : ax)), py = (float)(j + (swap ? by : ay)), pz = (float)(k + (swap ? bz : az));
    out[0] = (px + t * (float)(bx - ax) * (swap ? -1.0f : 1.0f)) * sx;
    out[1] = (py + t * (float)(by - ay) * (swap ? -1.0f : 1.0f)) * sy;
    out[2] = (pz + t * (float)(bz - az) * (swap ? -1.0f : 1.0f)) * sz;
}

__global__ void mc_emit_kernel(const float *__restrict__ v, int nx, int ny, int nz, float level, float sx, float sy,
                               float sz, const McTable T, const long long *__restrict__ block_off, float *tris) {
    const long long ncell = (long long)(nx - 1) * (ny - 1) * (nz - 1);
    const long long id = blockIdx.x * (long long)kMcBlock + threadIdx.x;
    int n = 0, cs = 0, i = 0, j = 0, k = 0;
    float c[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (id < ncell) {
        k = (int)(id % (nz - 1));
        j = (int)((id / (nz - 1)) % (ny - 1));
        i = (int)(id / ((long long)(nz - 1) * (ny - 1)));
        cs = mc_case(v, i, j, k, ny, nz, level, c);
        n = T.ntri[cs];
    }
    // exclusive scan of n over the block, in cell order
    __shared__ int ws[kMcBlock / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int s = n;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, s, o);
        if (lane >= o) s += y;
    }
    if (lane == 31) ws[w] = s;
    __syncthreads();
    int before = 0;
    for (int q = 0; q < w; ++q) before += ws[q];
    const long long off = block_off[blockIdx.x] + before + s - n;
    float *o = tris + off * 9;
    int e0 = 0;
    for (int L = 0; L < T.nloop[cs]; ++L) {
        const int len = T.len[cs][L];
        float p[12][3];
        for (int t = 0; t < len; ++t) mc_vertex(T.edge[cs][e0 + t], i, j, k, c, level, sx, sy, sz, p[t]);
        if (len == 3) {
            for (int t = 0; t < 3; ++t)
                for (int d = 0; d < 3; ++d) o[3 * t + d] = p[t][d];
            o += 9;
        } else {
            float m[3] = {0.0f, 0.0f, 0.0f};
            for (int t = 0; t < len; ++t)
                for (int d = 0; d < 3; ++d) m[d] += p[t][d];
            for (int d = 0; d < 3; ++d) m[d] /= (float)len;
            for (int t = 0; t < len; ++t) {
                const int u = t + 1 < len ? t + 1 : 0;
                for (int d = 0; d < 3; ++d) {
                    o[d] = m[d];
                    o[3 + d] = p[t][d];
                    o[6 + d] = p[u][d];
                }
                o += 9;
            }
        }
        e0 += len;
    }
}

}  // namespace gbs

using namespace gbs;

static long long mc_blocks(int nx, int ny, int nz) {
    const long long ncell = (long long)(nx - 1) * (ny - 1) * (nz - 1);
    return (ncell + kMcBlock - 1) / kMcBlock;
}

extern "C" size_t gbsimp_marching_cubes_ws_bytes(int nx, int ny, int nz) {
    if (nx < 2 || ny < 2 || nz < 2) return 0;
    return (size_t)(mc_blocks(nx, ny, nz) + 1) * sizeof(long long) + 256;
}

extern "C" int gbsimp_marching_cubes_table(unsigned char *ntri, unsigned char *nloop, unsigned char *len,
                                           signed char *edge) {
    const McTable &T = mc_table();
    if (ntri) memcpy(ntri, T.ntri, sizeof T.ntri);
    if (nloop) memcpy(nloop, T.nloop, sizeof T.nloop);
    if (len) memcpy(len, T.len, sizeof T.len);
    if (edge) memcpy(edge, T.edge, sizeof T.edge);
    return kMcMaxTri;
}

extern "C" int gbsimp_marching_cubes(gbsimp_ctx *ctx, int nx, int ny, int nz, const float *vol, double level,
                                     double sx, double sy, double sz, float *tris, int64_t max_tris,
                                     int64_t *n_tris, void *ws, size_t ws_bytes, void *stream) {
    if (!ctx || !vol || !n_tris || !ws || nx < 2 || ny < 2 || nz < 2 || max_tris < 0 || !isfinite(level))
        return set_error(GBS_EINVAL, "gbsimp_marching_cubes: bad arguments");
    if ((long long)nx * ny * nz > (1LL << 31)) return set_error(GBS_EINVAL, "gbsimp_marching_cubes: grid too large");
    if (ws_bytes < gbsimp_marching_cubes_ws_bytes(nx, ny, nz))
        return set_error(GBS_EINVAL, "gbsimp_marching_cubes: workspace too small");
    cudaStream_t st = (cudaStream_t)stream;
    const McTable &T = mc_table();
    const long long nb = mc_blocks(nx, ny, nz);
    long long *blk = (long long *)(((uintptr_t)ws + 255) & ~(uintptr_t)255);
    mc_count_kernel<<<(unsigned)nb, kMcBlock, 0, st>>>(vol, nx, ny, nz, (float)level, T, blk);
    GBS_LAUNCH_CHECK("mc_count_kernel");
    mc_scan_kernel<<<1, 1024, 0, st>>>(blk, nb);
    GBS_LAUNCH_CHECK("mc_scan_kernel");
    void *hp = thread_pinned();
    if (!hp) return set_error(GBS_ECUDA, "no pinned staging buffer");
    GBS_CUDA_TRY(cudaMemcpyAsync(hp, blk + nb, sizeof(long long), cudaMemcpyDeviceToHost, st));
    GBS_CUDA_TRY(cudaStreamSynchronize(st));
    long long total = 0;
    memcpy(&total, hp, sizeof total);
    *n_tris = total;
    if (!tris || total > max_tris || total == 0) return GBS_OK;  // size query
    mc_emit_kernel<<<(unsigned)nb, kMcBlock, 0, st>>>(vol, nx, ny, nz, (float)level, (float)sx, (float)sy, (float)sz,
                                                      T, blk, tris);
    GBS_LAUNCH_CHECK("mc_emit_kernel");
    return GBS_OK;
}
