// anl_mc.cu -- the iso-surface export of a density field: marching cubes as stream compaction.
//
// Replaces export.surface (export.py:121-147): np.pad by one element, ndimage.zoom(order=1)
// by `upsample`, skimage.measure.marching_cubes at `level`, trimesh Taubin smoothing and the
// fragment split. On the GPU:
//  1. k_mc_zoom: the padded, linearly upsampled sample grid (ndimage.zoom's mapping
//     o -> o (n_in - 1) / (n_out - 1) per axis);
//  2. k_mc_classify: per sample, the cube case of the cell it is the low corner of, the
//     number of triangles of that case, and which of its 3 forward edges cross the level;
//  3. an exclusive scan of (vertices, triangles) per sample gives every crossing edge its
//     vertex index and every cell its first triangle (stream compaction, no atomics);
//  4. k_mc_emit: vertices interpolated on their edges, triangles written through the table.
// Vertices belong to grid edges, so the mesh is indexed and closed (the field is padded by
// zeros). The case table is derived, not tabulated: per face, the crossing points are joined
// so that inside corners (value > level) on a face's diagonal stay separated; segments are
// oriented with the inside on their left seen from outside the cube and chained into loops,
// which are fanned into triangles facing away from the inside. Both cubes sharing a face see
// the same segments, which makes the surface watertight.
// Taubin smoothing (lambda | mu, equal-weight umbrella operator) and the connected components
// run on the same device mesh.
#include <algorithm>
#include <cstring>
#include <new>
#include <vector>

#include "anl_common.cuh"
#include "anl_scan.cuh"

namespace anl {

// ------------------------------------------------------------------ case table (host)

constexpr int MC_MAXTRI = 8;

struct McTable {
    uint8_t ntri[256];
    int8_t tri[256][MC_MAXTRI * 3];  // cube edges: e = 4 * axis + q
};

// Cube corners c: bits (x, y, z). Edge e = 4 a + q along axis a; q packs the other two bits in
// increasing axis order. Its low corner has bit a = 0.
static int mc_edge_corner(int e) {
    const int a = e >> 2, q = e & 3;
    const int o1 = a == 0 ? 1 : 0, o2 = a == 2 ? 1 : 2;
    return ((q & 1) << o1) | (((q >> 1) & 1) << o2);
}
static int mc_edge_id(int a, int c) {  // edge along axis a starting at corner c (bit a clear)
    const int o1 = a == 0 ? 1 : 0, o2 = a == 2 ? 1 : 2;
    return 4 * a + ((c >> o1) & 1) + 2 * ((c >> o2) & 1);
}

// edges e and f lie on a common face of the cube
static bool mc_share_face(int e, int f) {
    auto faces = [](int x, int* fa) {  // the two faces (axis * 2 + side) of edge x
        const int a = x >> 2, q = x & 3;
        const int o1 = a == 0 ? 1 : 0, o2 = a == 2 ? 1 : 2;
        fa[0] = 2 * o1 + (q & 1);
        fa[1] = 2 * o2 + ((q >> 1) & 1);
    };
    int fe[2], ff[2];
    faces(e, fe);
    faces(f, ff);
    return fe[0] == ff[0] || fe[0] == ff[1] || fe[1] == ff[0] || fe[1] == ff[1];
}

static bool mc_build_table(McTable* T) {
    std::memset(T, 0, sizeof(McTable));
    for (int cs = 0; cs < 256; ++cs) {
        auto in = [&](int c) { return (cs >> c) & 1; };
        auto pos = [](int c, double* p) {
            p[0] = c & 1;
            p[1] = (c >> 1) & 1;
            p[2] = (c >> 2) & 1;
        };
        auto mid = [&](int e, double* p) {
            pos(mc_edge_corner(e), p);
            p[e >> 2] += 0.5;
        };
        int next[12];
        for (int e = 0; e < 12; ++e) next[e] = -1;
        int nseg = 0;
        for (int a = 0; a < 3; ++a)
            for (int s = 0; s < 2; ++s) {
                const int b = a == 0 ? 1 : 0, d = a == 2 ? 1 : 2;
                // corners around the face in cyclic order, and the edge from corner k to k+1
                int cc[4], ee[4];
                const int bits[4][2] = {{0, 0}, {1, 0}, {1, 1}, {0, 1}};
                for (int k = 0; k < 4; ++k) cc[k] = (s << a) | (bits[k][0] << b) | (bits[k][1] << d);
                for (int k = 0; k < 4; ++k) {
                    const int c0 = cc[k], c1 = cc[(k + 1) & 3];
                    const int ax = (c0 ^ c1) == (1 << b) ? b : d;
                    ee[k] = mc_edge_id(ax, c0 & c1);
                }
                int cross[4], nc = 0;
                for (int k = 0; k < 4; ++k)
                    if (in(cc[k]) != in(cc[(k + 1) & 3])) cross[nc++] = k;
                if (nc == 0) continue;
                // segments (edge pair) with the inside corner they cut off or border
                int seg[2][2], test[2], ns = 0;
                if (nc == 2) {
                    seg[0][0] = ee[cross[0]];
                    seg[0][1] = ee[cross[1]];
                    test[0] = -1;
                    for (int k = 0; k < 4; ++k)
                        if (in(cc[k])) test[0] = cc[k];
                    ns = 1;
                } else {  // 4 crossings: inside corners on one diagonal, each cut off alone
                    for (int k = 0; k < 4; ++k)
                        if (in(cc[k])) {
                            seg[ns][0] = ee[(k + 3) & 3];  // edge arriving at corner k
                            seg[ns][1] = ee[k];            // edge leaving corner k
                            test[ns] = cc[k];
                            ++ns;
                        }
                }
                double n[3] = {0, 0, 0};
                n[a] = s ? 1.0 : -1.0;
                for (int g = 0; g < ns; ++g) {
                    double p[3], q[3], t[3];
                    mid(seg[g][0], p);
                    mid(seg[g][1], q);
                    pos(test[g], t);
                    const double u[3] = {q[0] - p[0], q[1] - p[1], q[2] - p[2]};
                    const double x[3] = {u[1] * n[2] - u[2] * n[1], u[2] * n[0] - u[0] * n[2], u[0] * n[1] - u[1] * n[0]};
                    double dot = 0;
                    for (int k = 0; k < 3; ++k) dot += x[k] * (t[k] - 0.5 * (p[k] + q[k]));
                    int e0 = seg[g][0], e1 = seg[g][1];
                    if (dot < 0) std::swap(e0, e1);
                    if (next[e0] != -1) return false;  // each crossing edge starts one segment
                    next[e0] = e1;
                    ++nseg;
                }
            }
        // chain into loops and fan them
        bool used[12] = {};
        int nt = 0;
        for (int e = 0; e < 12; ++e) {
            if (next[e] < 0 || used[e]) continue;
            int loop[12], len = 0, cur = e;
            while (!used[cur]) {
                if (next[cur] < 0 || len >= 12) return false;
                used[cur] = true;
                loop[len++] = cur;
                cur = next[cur];
            }
            if (cur != e || len < 3) return false;
            // fan apex: the first position whose diagonals join no two edges of a common cube
            // face (a diagonal on a face would also be drawn by the cube across it)
            int apex = -1;
            for (int i = 0; i < len && apex < 0; ++i) {
                bool ok = true;
                for (int k = 0; k < len && ok; ++k)
                    if (k != i && k != (i + 1) % len && k != (i + len - 1) % len && mc_share_face(loop[i], loop[k]))
                        ok = false;
                if (ok) apex = i;
            }
            if (apex < 0) return false;
            for (int k = 1; k + 1 < len; ++k) {
                if (nt >= MC_MAXTRI) return false;
                T->tri[cs][3 * nt] = (int8_t)loop[apex];
                T->tri[cs][3 * nt + 1] = (int8_t)loop[(apex + k) % len];
                T->tri[cs][3 * nt + 2] = (int8_t)loop[(apex + k + 1) % len];
                ++nt;
            }
        }
        T->ntri[cs] = (uint8_t)nt;
        (void)nseg;
    }
    return true;
}

static const McTable* mc_table() {
    static McTable table;
    static const bool ok = mc_build_table(&table);  // built once, thread-safe
    return ok ? &table : nullptr;
}

// ------------------------------------------------------------------ device helpers

struct Grid3 {
    int nx, ny, nz;  // samples
    __host__ __device__ int64_t n() const { return (int64_t)nx * ny * nz; }
};

constexpr int MC_T = 256;

// padded element field: element (i-1, j-1, k-1) for 1 <= i <= nx etc., zero elsewhere
__device__ __forceinline__ float padded(const float* f, int nx, int ny, int nz, int i, int j, int k) {
    if (i < 1 || j < 1 || k < 1 || i > nx || j > ny || k > nz) return 0.f;
    return f[(int64_t)(i - 1) + (int64_t)nx * ((int64_t)(j - 1) + (int64_t)ny * (k - 1))];
}

// sample o of an axis zoomed from n_in to n_out points: the low input index and its weight
__device__ __forceinline__ void zoom_coord(int o, int n_in, int n_out, int& i0, float& w) {
    if (n_out == n_in) {
        i0 = o;
        w = 0.f;
        return;
    }
    const double x = (double)o * (double)(n_in - 1) / (double)(n_out - 1);
    int i = (int)floor(x);
    if (i > n_in - 2) i = n_in - 2;
    if (i < 0) i = 0;
    i0 = i;
    w = (float)(x - (double)i);
}

__global__ void k_mc_zoom(const float* f, int nx, int ny, int nz, Grid3 G, float* g) {
    const int px = nx + 2, py = ny + 2, pz = nz + 2;
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < G.n(); s += (int64_t)gridDim.x * blockDim.x) {
        const int I = (int)(s % G.nx), J = (int)((s / G.nx) % G.ny), K = (int)(s / ((int64_t)G.nx * G.ny));
        int i0, j0, k0;
        float wx, wy, wz;
        zoom_coord(I, px, G.nx, i0, wx);
        zoom_coord(J, py, G.ny, j0, wy);
        zoom_coord(K, pz, G.nz, k0, wz);
        float acc = 0.f;
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            const int di = c & 1, dj = (c >> 1) & 1, dk = (c >> 2) & 1;
            const float w = (di ? wx : 1.f - wx) * (dj ? wy : 1.f - wy) * (dk ? wz : 1.f - wz);
            if (w != 0.f) acc += w * padded(f, nx, ny, nz, i0 + di, j0 + dj, k0 + dk);
        }
        g[s] = acc;
    }
}

// code[s] = cube case of the cell whose low corner is s (0 if s is on a high face) | crossing
// mask of the 3 forward edges << 8; cnt[s] = (vertices, triangles) owned by s
__global__ void k_mc_classify(const float* g, Grid3 G, float level, const uint8_t* ntri, uint16_t* code, int2* cnt) {
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < G.n(); s += (int64_t)gridDim.x * blockDim.x) {
        const int I = (int)(s % G.nx), J = (int)((s / G.nx) % G.ny), K = (int)(s / ((int64_t)G.nx * G.ny));
        const int64_t sx = 1, sy = G.nx, sz = (int64_t)G.nx * G.ny;
        const bool v0 = g[s] > level;
        int mask = 0;
        if (I + 1 < G.nx && (g[s + sx] > level) != v0) mask |= 1;
        if (J + 1 < G.ny && (g[s + sy] > level) != v0) mask |= 2;
        if (K + 1 < G.nz && (g[s + sz] > level) != v0) mask |= 4;
        int cs = 0, nt = 0;
        if (I + 1 < G.nx && J + 1 < G.ny && K + 1 < G.nz) {
#pragma unroll
            for (int c = 0; c < 8; ++c) {
                const int64_t o = (c & 1) * sx + ((c >> 1) & 1) * sy + ((c >> 2) & 1) * sz;
                if (g[s + o] > level) cs |= 1 << c;
            }
            nt = __ldg(ntri + cs);
        }
        code[s] = (uint16_t)(cs | (mask << 8));
        cnt[s] = make_int2(__popc(mask), nt);
    }
}

__global__ void k_mc_emit(const float* g, Grid3 G, float level, const uint16_t* code, const int2* off,
                          const uint8_t* ntri, const int8_t* tri, float3 spacing, float3 origin, float* verts,
                          int* faces) {
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < G.n(); s += (int64_t)gridDim.x * blockDim.x) {
        const uint16_t cd = code[s];
        const int mask = cd >> 8, cs = cd & 255;
        const int I = (int)(s % G.nx), J = (int)((s / G.nx) % G.ny), K = (int)(s / ((int64_t)G.nx * G.ny));
        const int64_t st[3] = {1, G.nx, (int64_t)G.nx * G.ny};
        const int2 o = off[s];
        if (mask) {
            const float f0 = g[s];
            int v = o.x;
            for (int a = 0; a < 3; ++a) {
                if (!((mask >> a) & 1)) continue;
                const float f1 = g[s + st[a]];
                const float t = (level - f0) / (f1 - f0);
                float p[3] = {(float)I, (float)J, (float)K};
                p[a] += t;
                verts[3 * (int64_t)v] = origin.x + spacing.x * p[0];
                verts[3 * (int64_t)v + 1] = origin.y + spacing.y * p[1];
                verts[3 * (int64_t)v + 2] = origin.z + spacing.z * p[2];
                ++v;
            }
        }
        const int nt = (I + 1 < G.nx && J + 1 < G.ny && K + 1 < G.nz) ? __ldg(ntri + cs) : 0;
        for (int t = 0; t < nt; ++t)
            for (int q = 0; q < 3; ++q) {
                const int e = tri[cs * MC_MAXTRI * 3 + 3 * t + q];
                const int a = e >> 2, qq = e & 3;
                const int o1 = a == 0 ? 1 : 0, o2 = a == 2 ? 1 : 2;
                const int64_t sc = s + (qq & 1) * st[o1] + ((qq >> 1) & 1) * st[o2];
                const int m = code[sc] >> 8;
                faces[3 * ((int64_t)o.y + t) + q] = off[sc].x + __popc(m & ((1 << a) - 1));
            }
    }
}

// ------------------------------------------------------------------ smoothing and components

// incidences: for every (face, corner) the vertex it belongs to
__global__ void k_inc_count(int64_t nf, const int* faces, int* cnt) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < 3 * nf; t += (int64_t)gridDim.x * blockDim.x)
        atomicAdd(cnt + faces[t], 1);
}
__global__ void k_inc_fill(int64_t nf, const int* faces, const int* off, int* fillc, int* inc) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < 3 * nf; t += (int64_t)gridDim.x * blockDim.x) {
        const int v = faces[t];
        inc[off[v] + atomicAdd(fillc + v, 1)] = (int)t;
    }
}
// each vertex's incidence list in increasing order (the fill above is unordered)
__global__ void k_inc_sort(int64_t nv, const int* off, const int* cnt, int* inc) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < nv; v += (int64_t)gridDim.x * blockDim.x) {
        int* l = inc + off[v];
        const int m = cnt[v];
        for (int i = 1; i < m; ++i) {
            const int x = l[i];
            int j = i - 1;
            while (j >= 0 && l[j] > x) {
                l[j + 1] = l[j];
                --j;
            }
            l[j + 1] = x;
        }
    }
}

// one Taubin half-step: v' = v + w (mean of the neighbours - v). On a closed, consistently
// oriented mesh every neighbour of a vertex follows it in exactly one of its faces.
__global__ void k_taubin(int64_t nv, const int* faces, const int* off, const int* cnt, const int* inc, const float* vin,
                         float w, float* vout) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < nv; v += (int64_t)gridDim.x * blockDim.x) {
        const int m = cnt[v];
        const float px = vin[3 * v], py = vin[3 * v + 1], pz = vin[3 * v + 2];
        if (m == 0) {
            vout[3 * v] = px;
            vout[3 * v + 1] = py;
            vout[3 * v + 2] = pz;
            continue;
        }
        float sx = 0.f, sy = 0.f, sz = 0.f;
        for (int q = 0; q < m; ++q) {
            const int t = inc[off[v] + q];
            const int f = t / 3, c = t - 3 * f;
            const int nb = faces[3 * f + (c + 1) % 3];
            sx += vin[3 * (int64_t)nb];
            sy += vin[3 * (int64_t)nb + 1];
            sz += vin[3 * (int64_t)nb + 2];
        }
        const float inv = 1.f / (float)m;
        vout[3 * v] = px + w * (sx * inv - px);
        vout[3 * v + 1] = py + w * (sy * inv - py);
        vout[3 * v + 2] = pz + w * (sz * inv - pz);
    }
}

// connected components: labels only decrease (to the smallest vertex of the component)
__global__ void k_cc_init(int64_t nv, int* lab) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < nv; v += (int64_t)gridDim.x * blockDim.x)
        lab[v] = (int)v;
}
__global__ void k_cc_hook(int64_t nf, const int* faces, int* lab, int* changed) {
    for (int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; f < nf; f += (int64_t)gridDim.x * blockDim.x) {
        const int a = lab[faces[3 * f]], b = lab[faces[3 * f + 1]], c = lab[faces[3 * f + 2]];
        const int m = min(a, min(b, c));
        if (a != m) {
            atomicMin(lab + a, m);
            *changed = 1;
        }
        if (b != m) {
            atomicMin(lab + b, m);
            *changed = 1;
        }
        if (c != m) {
            atomicMin(lab + c, m);
            *changed = 1;
        }
    }
}
__global__ void k_cc_jump(int64_t nv, int* lab) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < nv; v += (int64_t)gridDim.x * blockDim.x) {
        int l = lab[v];
        for (int k = 0; k < 64; ++k) {  // bounded pointer jumping
            const int p = lab[l];
            if (p == l) break;
            l = p;
        }
        lab[v] = l;
    }
}
__global__ void k_cc_face(int64_t nf, const int* faces, const int* lab, int* flab) {
    for (int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; f < nf; f += (int64_t)gridDim.x * blockDim.x)
        flab[f] = lab[faces[3 * f]];
}

static int vgrid_mc(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>(4 * 1216, (n + MC_T - 1) / MC_T)); }

}  // namespace anl

// ------------------------------------------------------------------ the export handle

using namespace anl;

struct anl_mc {
    // device buffers, grown on demand
    float* g = nullptr;
    size_t g_cap = 0;  // samples
    uint16_t* code = nullptr;
    size_t code_cap = 0;
    int2* cnt = nullptr;
    size_t cnt_cap = 0;
    int2* off = nullptr;
    size_t off_cap = 0;
    int2* part = nullptr;   // SCAN_BLOCKS
    int2* tot2 = nullptr;   // 1
    int* ipart = nullptr;   // SCAN_BLOCKS
    int* itot = nullptr;    // 1 + changed flag
    uint8_t* ntri = nullptr;
    int8_t* tri = nullptr;
    float* verts = nullptr;
    size_t v_cap = 0;
    float* verts2 = nullptr;
    size_t v2_cap = 0;
    int* faces = nullptr;
    size_t f_cap = 0;
    int* vcnt = nullptr;
    size_t vcnt_cap = 0;
    int* voff = nullptr;
    size_t voff_cap = 0;
    int* vfill = nullptr;
    size_t vfill_cap = 0;
    int* lab = nullptr;
    size_t lab_cap = 0;
    int* inc = nullptr;
    size_t inc_cap = 0;
    int* host = nullptr;  // pinned: totals and flags
    int64_t nv = 0, nf = 0;
    bool have_inc = false;
};

namespace {

void mc_free(anl_mc* m) {
    std::lock_guard<std::recursive_mutex> lock(device_sync_mutex());
    cudaFree(m->g);
    cudaFree(m->code);
    cudaFree(m->cnt);
    cudaFree(m->off);
    cudaFree(m->part);
    cudaFree(m->tot2);
    cudaFree(m->ipart);
    cudaFree(m->itot);
    cudaFree(m->ntri);
    cudaFree(m->tri);
    cudaFree(m->verts);
    cudaFree(m->verts2);
    cudaFree(m->faces);
    cudaFree(m->vcnt);
    cudaFree(m->voff);
    cudaFree(m->vfill);
    cudaFree(m->lab);
    cudaFree(m->inc);
    if (m->host) cudaFreeHost(m->host);
    delete m;
}

cudaStream_t S(anl_stream_t s) { return (cudaStream_t)s; }

}  // namespace

extern "C" {

int anl_mc_create(anl_mc** out) {
    if (!out) {
        set_error("anl_mc_create: null argument");
        return ANL_ERR_BADARG;
    }
    *out = nullptr;
    const McTable* T = mc_table();
    if (!T) {
        set_error("marching-cubes case table construction failed");
        return ANL_ERR_BADARG;
    }
    anl_mc* m = new (std::nothrow) anl_mc();
    if (!m) return ANL_ERR_NOMEM;
    if (cudaMalloc((void**)&m->part, SCAN_BLOCKS * sizeof(int2)) != cudaSuccess ||
        cudaMalloc((void**)&m->tot2, sizeof(int2)) != cudaSuccess ||
        cudaMalloc((void**)&m->ipart, SCAN_BLOCKS * sizeof(int)) != cudaSuccess ||
        cudaMalloc((void**)&m->itot, 4 * sizeof(int)) != cudaSuccess ||
        cudaMalloc((void**)&m->ntri, sizeof(T->ntri)) != cudaSuccess ||
        cudaMalloc((void**)&m->tri, sizeof(T->tri)) != cudaSuccess ||
        cudaMallocHost((void**)&m->host, 8 * sizeof(int)) != cudaSuccess) {
        cudaGetLastError();
        set_error("anl_mc_create: allocation failed");
        mc_free(m);
        return ANL_ERR_NOMEM;
    }
    if (cudaMemcpy(m->ntri, T->ntri, sizeof(T->ntri), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(m->tri, T->tri, sizeof(T->tri), cudaMemcpyHostToDevice) != cudaSuccess) {
        set_error("anl_mc_create: table upload failed");
        mc_free(m);
        return ANL_ERR_CUDA;
    }
    *out = m;
    return ANL_OK;
}

void anl_mc_destroy(anl_mc* m) {
    if (m) mc_free(m);
}

int anl_mc_table(uint8_t* ntri_h, int8_t* tri_h) {
    const McTable* T = mc_table();
    if (!T || !ntri_h || !tri_h) {
        set_error("anl_mc_table: %s", T ? "null argument" : "table construction failed");
        return ANL_ERR_BADARG;
    }
    std::memcpy(ntri_h, T->ntri, sizeof(T->ntri));
    std::memcpy(tri_h, T->tri, sizeof(T->tri));
    return ANL_OK;
}

int anl_mc_extract(anl_mc* m, const float* field, int nx, int ny, int nz, int upsample, double level, double h,
                   const double* origin_h, int64_t* nverts_h, int64_t* nfaces_h, anl_stream_t stream) {
    if (!m || !field || !origin_h || !nverts_h || !nfaces_h || nx < 1 || ny < 1 || nz < 1 || upsample < 1 ||
        upsample > 8 || !(h > 0)) {
        set_error("anl_mc_extract: bad argument");
        return ANL_ERR_BADARG;
    }
    cudaStream_t s = S(stream);
    const int px = nx + 2, py = ny + 2, pz = nz + 2;
    const Grid3 G{px * upsample, py * upsample, pz * upsample};
    const int64_t n = G.n();
    if (n > ((int64_t)1 << 29)) {  // 3 vertices per sample must fit the int32 indices
        set_error("anl_mc_extract: %lld samples exceed the 2^29 limit", (long long)n);
        return ANL_ERR_BADARG;
    }
    ANL_TRY(grow(m->g, m->g_cap, n, sizeof(float)));
    ANL_TRY(grow(m->code, m->code_cap, n, sizeof(uint16_t)));
    ANL_TRY(grow(m->cnt, m->cnt_cap, n, sizeof(int2)));
    ANL_TRY(grow(m->off, m->off_cap, n, sizeof(int2)));
    k_mc_zoom<<<vgrid_mc(n), MC_T, 0, s>>>(field, nx, ny, nz, G, m->g);
    ANL_LAUNCH_CHECK();
    k_mc_classify<<<vgrid_mc(n), MC_T, 0, s>>>(m->g, G, (float)level, m->ntri, m->code, m->cnt);
    ANL_LAUNCH_CHECK();
    ANL_TRY(scan_exclusive<int2>(m->cnt, n, m->off, m->part, m->tot2, s));
    ANL_CUDA(cudaMemcpyAsync(m->host, m->tot2, sizeof(int2), cudaMemcpyDeviceToHost, s));
    ANL_CUDA(cudaStreamSynchronize(s));
    const int64_t nv = m->host[0], nf = m->host[1];
    ANL_TRY(grow(m->verts, m->v_cap, 3 * nv, sizeof(float)));
    ANL_TRY(grow(m->verts2, m->v2_cap, 3 * nv, sizeof(float)));
    ANL_TRY(grow(m->faces, m->f_cap, 3 * nf, sizeof(int)));
    // sample spacing (export.py:126) and the shift of export.py:131 (padded index p sits at
    // origin + (p - 0.5) h)
    const float3 sp = make_float3((float)(h * (px - 1) / (G.nx - 1)), (float)(h * (py - 1) / (G.ny - 1)),
                                  (float)(h * (pz - 1) / (G.nz - 1)));
    const float3 org = make_float3((float)(origin_h[0] - 0.5 * h), (float)(origin_h[1] - 0.5 * h),
                                   (float)(origin_h[2] - 0.5 * h));
    k_mc_emit<<<vgrid_mc(n), MC_T, 0, s>>>(m->g, G, (float)level, m->code, m->off, m->ntri, m->tri, sp, org, m->verts,
                                           m->faces);
    ANL_LAUNCH_CHECK();
    m->nv = nv;
    m->nf = nf;
    m->have_inc = false;
    *nverts_h = nv;
    *nfaces_h = nf;
    return ANL_OK;
}

static int mc_incidence(anl_mc* m, cudaStream_t s) {
    if (m->have_inc) return ANL_OK;
    const int64_t nv = m->nv, nf = m->nf;
    ANL_TRY(grow(m->vcnt, m->vcnt_cap, nv, sizeof(int)));
    ANL_TRY(grow(m->voff, m->voff_cap, nv, sizeof(int)));
    ANL_TRY(grow(m->vfill, m->vfill_cap, nv, sizeof(int)));
    ANL_TRY(grow(m->lab, m->lab_cap, nv, sizeof(int)));
    ANL_TRY(grow(m->inc, m->inc_cap, 3 * nf, sizeof(int)));
    ANL_CUDA(cudaMemsetAsync(m->vcnt, 0, nv * sizeof(int), s));
    ANL_CUDA(cudaMemsetAsync(m->vfill, 0, nv * sizeof(int), s));
    k_inc_count<<<vgrid_mc(3 * nf), MC_T, 0, s>>>(nf, m->faces, m->vcnt);
    ANL_LAUNCH_CHECK();
    ANL_TRY(scan_exclusive<int>(m->vcnt, nv, m->voff, m->ipart, m->itot, s));
    k_inc_fill<<<vgrid_mc(3 * nf), MC_T, 0, s>>>(nf, m->faces, m->voff, m->vfill, m->inc);
    ANL_LAUNCH_CHECK();
    k_inc_sort<<<vgrid_mc(nv), MC_T, 0, s>>>(nv, m->voff, m->vcnt, m->inc);
    ANL_LAUNCH_CHECK();
    m->have_inc = true;
    return ANL_OK;
}

int anl_mc_smooth(anl_mc* m, int iterations, double lamb, double mu, anl_stream_t stream) {
    if (!m || iterations < 0) {
        set_error("anl_mc_smooth: bad argument");
        return ANL_ERR_BADARG;
    }
    if (m->nv == 0 || iterations == 0) return ANL_OK;
    cudaStream_t s = S(stream);
    ANL_TRY(mc_incidence(m, s));
    for (int it = 0; it < iterations; ++it) {
        const float w = (float)(it % 2 == 0 ? lamb : mu);
        k_taubin<<<vgrid_mc(m->nv), MC_T, 0, s>>>(m->nv, m->faces, m->voff, m->vcnt, m->inc, m->verts, w, m->verts2);
        ANL_LAUNCH_CHECK();
        std::swap(m->verts, m->verts2);
    }
    return ANL_OK;
}

int anl_mc_components(anl_mc* m, int32_t* face_label, int* ncomp_iters_h, anl_stream_t stream) {
    if (!m || !face_label) {
        set_error("anl_mc_components: null argument");
        return ANL_ERR_BADARG;
    }
    if (m->nf == 0) return ANL_OK;
    cudaStream_t s = S(stream);
    ANL_TRY(mc_incidence(m, s));
    k_cc_init<<<vgrid_mc(m->nv), MC_T, 0, s>>>(m->nv, m->lab);
    ANL_LAUNCH_CHECK();
    int it = 0;
    for (; it < 256; ++it) {
        ANL_CUDA(cudaMemsetAsync(m->itot + 1, 0, sizeof(int), s));
        k_cc_hook<<<vgrid_mc(m->nf), MC_T, 0, s>>>(m->nf, m->faces, m->lab, m->itot + 1);
        ANL_LAUNCH_CHECK();
        k_cc_jump<<<vgrid_mc(m->nv), MC_T, 0, s>>>(m->nv, m->lab);
        ANL_LAUNCH_CHECK();
        ANL_CUDA(cudaMemcpyAsync(m->host + 2, m->itot + 1, sizeof(int), cudaMemcpyDeviceToHost, s));
        ANL_CUDA(cudaStreamSynchronize(s));
        if (m->host[2] == 0) break;
    }
    if (it == 256) {
        set_error("connected components did not settle in 256 rounds");
        return ANL_ERR_MAXITER;
    }
    k_cc_face<<<vgrid_mc(m->nf), MC_T, 0, s>>>(m->nf, m->faces, m->lab, face_label);
    ANL_LAUNCH_CHECK();
    if (ncomp_iters_h) *ncomp_iters_h = it + 1;
    return ANL_OK;
}

int anl_mc_copy(anl_mc* m, float* verts, int32_t* faces, anl_stream_t stream) {
    if (!m || (m->nv > 0 && !verts) || (m->nf > 0 && !faces)) {
        set_error("anl_mc_copy: null argument");
        return ANL_ERR_BADARG;
    }
    cudaStream_t s = S(stream);
    if (m->nv) ANL_CUDA(cudaMemcpyAsync(verts, m->verts, 3 * m->nv * sizeof(float), cudaMemcpyDefault, s));
    if (m->nf) ANL_CUDA(cudaMemcpyAsync(faces, m->faces, 3 * m->nf * sizeof(int), cudaMemcpyDefault, s));
    return ANL_OK;
}

}  // extern "C"
