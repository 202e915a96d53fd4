// anl_nn.cu -- the layers of the warm-start network: 3D convolution (forward, backward with
// respect to data and weights), GELU, 2x average pooling, 2x nearest upsampling, a masked
// mean-squared error and Adam. No counterpart in the reference: the network predicts the
// initial guess that the reference takes from the previous SIMP iterate (optimize.py:122).
//
// Tensors are one sample, channel-major: [C][D][H][W] with W (x) fastest, FP32. Convolutions
// are 3x3x3 (zero padding 1) or 1x1x1, stride 1. Gradients are deterministic: the weight
// gradient sums per-chunk partials in a fixed order, nothing depends on atomics.
#include <algorithm>

#include "anl_common.cuh"

namespace anl {

constexpr int NN_TX = 8, NN_TY = 8, NN_TZ = 4;  // output voxel tile of a conv CTA
constexpr int NN_T = NN_TX * NN_TY * NN_TZ;     // threads: one voxel each
constexpr int NN_CO = 16;                       // output channels per CTA

__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.f + erff(z * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float z) {
    return 0.5f * (1.f + erff(z * 0.70710678118654752f)) + z * 0.39894228040143268f * expf(-0.5f * z * z);
}

// z = conv(x, w) + b; a = gelu(z) when `act` (a may be null otherwise). w: [cout][cin][K^3].
template <int K>
__global__ void __launch_bounds__(NN_T) k_conv3d(const float* __restrict__ x, const float* __restrict__ w,
                                                 const float* __restrict__ b, float* z, float* a, int cin, int cout,
                                                 int D, int H, int W, int act, int accumulate) {
    constexpr int R = K / 2;
    constexpr int SX = NN_TX + 2 * R, SY = NN_TY + 2 * R, SZ = NN_TZ + 2 * R;
    constexpr int KK = K * K * K;
    __shared__ float sx[SZ * SY * SX];
    __shared__ __align__(16) float sw[KK][NN_CO];
    const int tx = threadIdx.x % NN_TX, ty = (threadIdx.x / NN_TX) % NN_TY, tz = threadIdx.x / (NN_TX * NN_TY);
    const int gx = (W + NN_TX - 1) / NN_TX, gy = (H + NN_TY - 1) / NN_TY;
    const int bx = blockIdx.x % gx, by = (blockIdx.x / gx) % gy, bz = blockIdx.x / (gx * gy);
    const int x0 = bx * NN_TX, y0 = by * NN_TY, z0 = bz * NN_TZ;
    const int co0 = blockIdx.y * NN_CO;
    const int X = x0 + tx, Y = y0 + ty, Z = z0 + tz;
    const int64_t vol = (int64_t)D * H * W;
    float acc[NN_CO];
#pragma unroll
    for (int o = 0; o < NN_CO; ++o) acc[o] = 0.f;
    for (int ci = 0; ci < cin; ++ci) {
        const float* xc = x + (int64_t)ci * vol;
        for (int t = threadIdx.x; t < SZ * SY * SX; t += NN_T) {
            const int sxi = t % SX, syi = (t / SX) % SY, szi = t / (SX * SY);
            const int gxx = x0 - R + sxi, gyy = y0 - R + syi, gzz = z0 - R + szi;
            float v = 0.f;
            if (gxx >= 0 && gxx < W && gyy >= 0 && gyy < H && gzz >= 0 && gzz < D)
                v = xc[(int64_t)gzz * H * W + (int64_t)gyy * W + gxx];
            sx[t] = v;
        }
        for (int t = threadIdx.x; t < KK * NN_CO; t += NN_T) {
            const int o = t / KK, k = t - o * KK;
            const int co = co0 + o;
            sw[k][o] = co < cout ? w[((int64_t)co * cin + ci) * KK + k] : 0.f;
        }
        __syncthreads();
#pragma unroll 1
        for (int k = 0; k < KK; ++k) {
            const int kx = k % K, ky = (k / K) % K, kz = k / (K * K);
            const float xv = sx[((tz + kz) * SY + ty + ky) * SX + tx + kx];
            const float4* w4 = reinterpret_cast<const float4*>(&sw[k][0]);
#pragma unroll
            for (int q = 0; q < NN_CO / 4; ++q) {
                const float4 ww = w4[q];
                acc[4 * q] = fmaf(ww.x, xv, acc[4 * q]);
                acc[4 * q + 1] = fmaf(ww.y, xv, acc[4 * q + 1]);
                acc[4 * q + 2] = fmaf(ww.z, xv, acc[4 * q + 2]);
                acc[4 * q + 3] = fmaf(ww.w, xv, acc[4 * q + 3]);
            }
        }
        __syncthreads();
    }
    if (X >= W || Y >= H || Z >= D) return;
    const int64_t v = (int64_t)Z * H * W + (int64_t)Y * W + X;
#pragma unroll
    for (int o = 0; o < NN_CO; ++o) {
        const int co = co0 + o;
        if (co >= cout) break;
        const int64_t idx = (int64_t)co * vol + v;
        float zz = acc[o] + (b ? b[co] : 0.f);
        if (accumulate) zz += z[idx];
        z[idx] = zz;
        if (act) a[idx] = gelu(zz);
    }
}

// w'[ci][co][k] = w[co][ci][K^3 - 1 - k]: the weights of the transposed convolution
__global__ void k_flip_weights(const float* w, float* wt, int cin, int cout, int KK) {
    const int64_t n = (int64_t)cin * cout * KK;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        const int k = (int)(t % KK);
        const int64_t r = t / KK;
        const int co = (int)(r % cout), ci = (int)(r / cout);
        wt[t] = w[((int64_t)co * cin + ci) * KK + (KK - 1 - k)];
    }
}

// Weight and bias gradients, stage 1: CTA (voxel chunk c, input channel ci, output block)
// writes part[c][co][ci][k] = sum over its voxels of dz[co][v] x[ci][v + off(k)], and for
// ci == 0 also part_b[c][co] = sum dz[co][v]. Thread t < 16 K^3 owns (co, k).
template <int K>
__global__ void __launch_bounds__(512) k_conv3d_wgrad(const float* __restrict__ x, const float* __restrict__ dz, int cin,
                                                      int cout, int D, int H, int W, int64_t chunk, float* part,
                                                      float* part_b) {
    constexpr int R = K / 2, KK = K * K * K;
    constexpr int TV = 64;  // voxels staged per pass (a run along x)
    __shared__ float sdz[NN_CO][TV];
    __shared__ float sxh[TV + 2 * R][K * K];  // the x run with halo, for each (ky, kz) row
    const int co0 = blockIdx.z * NN_CO, ci = blockIdx.y, c = blockIdx.x;
    const int64_t vol = (int64_t)D * H * W;
    const int64_t v0 = (int64_t)c * chunk, v1 = min(vol, v0 + chunk);
    const int t = threadIdx.x;
    const int o = t / KK, k = t % KK;
    const bool own = t < NN_CO * KK;
    const int kx = k % K, ky = (k / K) % K, kz = k / (K * K);
    float acc = 0.f, accb = 0.f;
    const float* xc = x + (int64_t)ci * vol;
    // walk the chunk as runs of up to TV voxels within one x-row
    for (int64_t v = v0; v < v1;) {
        const int X = (int)(v % W);
        const int64_t row = v / W;
        const int Y = (int)(row % H), Z = (int)(row / H);
        const int n = (int)min((int64_t)(W - X), min((int64_t)TV, v1 - v));
        __syncthreads();
        for (int q = t; q < NN_CO * TV; q += blockDim.x) {
            const int oo = q / TV, i = q % TV;
            sdz[oo][i] = (i < n && co0 + oo < cout) ? dz[(int64_t)(co0 + oo) * vol + v + i] : 0.f;
        }
        for (int q = t; q < (TV + 2 * R) * K * K; q += blockDim.x) {
            const int i = q / (K * K), rr = q % (K * K);
            const int yy = Y + (rr % K) - R, zz = Z + (rr / K) - R, xx = X + i - R;
            float val = 0.f;
            if (i < n + 2 * R && xx >= 0 && xx < W && yy >= 0 && yy < H && zz >= 0 && zz < D)
                val = xc[(int64_t)zz * H * W + (int64_t)yy * W + xx];
            sxh[i][rr] = val;
        }
        __syncthreads();
        if (own) {
            const int rr = ky + K * kz;
            for (int i = 0; i < n; ++i) acc = fmaf(sdz[o][i], sxh[i + kx][rr], acc);
            if (k == 0)
                for (int i = 0; i < n; ++i) accb += sdz[o][i];
        }
        v += n;
    }
    if (own && co0 + o < cout) {
        part[(((int64_t)c * cout + co0 + o) * cin + ci) * KK + k] = acc;
        if (ci == 0 && k == 0) part_b[(int64_t)c * cout + co0 + o] = accb;
    }
}

// stage 2: dw = sum over chunks in order (accumulate into dw when `accumulate`)
__global__ void k_sum_parts(const float* part, int nchunk, int64_t n, float* out, int accumulate) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        float s = 0.f;
        for (int c = 0; c < nchunk; ++c) s += part[(int64_t)c * n + t];
        out[t] = accumulate ? out[t] + s : s;
    }
}

__global__ void k_gelu_bwd(int64_t n, const float* z, const float* da, float* dz) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
        dz[t] = da[t] * gelu_grad(z[t]);
}

// 2x average pooling per channel; D, H, W are the input (even) dims
__global__ void k_pool2(int64_t C, int D, int H, int W, const float* x, float* y) {
    const int d = D / 2, h = H / 2, w = W / 2;
    const int64_t n = C * d * h * w;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(t % w), j = (int)((t / w) % h), k = (int)((t / ((int64_t)w * h)) % d);
        const int64_t c = t / ((int64_t)w * h * d);
        const float* xc = x + c * D * H * W;
        float s = 0.f;
        for (int q = 0; q < 8; ++q)
            s += xc[(int64_t)(2 * k + (q >> 2)) * H * W + (int64_t)(2 * j + ((q >> 1) & 1)) * W + 2 * i + (q & 1)];
        y[t] = 0.125f * s;
    }
}
__global__ void k_pool2_bwd(int64_t C, int D, int H, int W, const float* dy, float* dx, int accumulate) {
    const int64_t n = C * D * H * W;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        const int X = (int)(t % W), Y = (int)((t / W) % H), Z = (int)((t / ((int64_t)W * H)) % D);
        const int64_t c = t / ((int64_t)W * H * D);
        const float g = 0.125f * dy[((c * (D / 2) + Z / 2) * (H / 2) + Y / 2) * (W / 2) + X / 2];
        dx[t] = accumulate ? dx[t] + g : g;
    }
}
// 2x nearest upsampling; D, H, W are the output dims
__global__ void k_up2(int64_t C, int D, int H, int W, const float* x, float* y) {
    const int64_t n = C * D * H * W;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        const int X = (int)(t % W), Y = (int)((t / W) % H), Z = (int)((t / ((int64_t)W * H)) % D);
        const int64_t c = t / ((int64_t)W * H * D);
        y[t] = x[((c * (D / 2) + Z / 2) * (H / 2) + Y / 2) * (W / 2) + X / 2];
    }
}
__global__ void k_up2_bwd(int64_t C, int D, int H, int W, const float* dy, float* dx) {
    const int d = D / 2, h = H / 2, w = W / 2;
    const int64_t n = C * d * h * w;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(t % w), j = (int)((t / w) % h), k = (int)((t / ((int64_t)w * h)) % d);
        const int64_t c = t / ((int64_t)w * h * d);
        const float* g = dy + c * D * H * W;
        float s = 0.f;
        for (int q = 0; q < 8; ++q)
            s += g[(int64_t)(2 * k + (q >> 2)) * H * W + (int64_t)(2 * j + ((q >> 1) & 1)) * W + 2 * i + (q & 1)];
        dx[t] = s;
    }
}

// masked MSE: loss = sum m (y - t)^2 / max(1, sum m) over C channels sharing the voxel mask;
// dy = 2 m (y - t) / max(1, sum m). Two-stage deterministic sums into out[0] (loss), out[1].
constexpr int NN_RT = 256;
__global__ void k_mse(int C, int64_t vol, const float* y, const float* tgt, const float* mask, float* dy,
                      double* partials, unsigned* counter, double* out) {
    __shared__ double sm[2 * NN_RT / 32];
    double v[2] = {0.0, 0.0};
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < vol; t += (int64_t)gridDim.x * blockDim.x) {
        const float m = mask[t];
        v[1] += m;
        for (int c = 0; c < C; ++c) {
            const float d = y[c * vol + t] - tgt[c * vol + t];
            v[0] += (double)(m * d * d);
        }
    }
    block_sum<2, NN_RT>(v, sm, threadIdx.x);
    finish_reduction<2, NN_RT>(v, blockIdx.x, gridDim.x, partials, counter, out, threadIdx.x, sm);
}
__global__ void k_mse_grad(int C, int64_t vol, const float* y, const float* tgt, const float* mask, const double* sums,
                           float* dy) {
    const float inv = (float)(1.0 / fmax(1.0, sums[1]));
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < (int64_t)C * vol;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t v = t % vol;
        dy[t] = 2.f * mask[v] * (y[t] - tgt[t]) * inv;
    }
}

__global__ void k_adam(int64_t n, float* p, const float* g, float* m, float* v, float lr, float b1, float b2, float eps,
                       float c1, float c2) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        const float gg = g[t];
        const float mm = b1 * m[t] + (1.f - b1) * gg;
        const float vv = b2 * v[t] + (1.f - b2) * gg * gg;
        m[t] = mm;
        v[t] = vv;
        p[t] -= lr * (mm / c1) / (sqrtf(vv / c2) + eps);
    }
}

static int grid1(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>(4 * 1216, (n + 255) / 256)); }

}  // namespace anl

using namespace anl;

extern "C" {

int anl_nn_conv3d(const float* x, const float* w, const float* b, float* z, float* a, int cin, int cout, int D, int H,
                  int W, int ksize, int act, int accumulate, anl_stream_t stream) {
    if (!x || !w || !z || (act && !a) || cin < 1 || cout < 1 || D < 1 || H < 1 || W < 1 || (ksize != 1 && ksize != 3)) {
        set_error("anl_nn_conv3d: bad argument");
        return ANL_ERR_BADARG;
    }
    const int gx = (W + NN_TX - 1) / NN_TX, gy = (H + NN_TY - 1) / NN_TY, gz = (D + NN_TZ - 1) / NN_TZ;
    dim3 grid(gx * gy * gz, (cout + NN_CO - 1) / NN_CO);
    cudaStream_t s = (cudaStream_t)stream;
    if (ksize == 3) k_conv3d<3><<<grid, NN_T, 0, s>>>(x, w, b, z, a, cin, cout, D, H, W, act, accumulate);
    else k_conv3d<1><<<grid, NN_T, 0, s>>>(x, w, b, z, a, cin, cout, D, H, W, act, accumulate);
    ANL_LAUNCH_CHECK();
    return ANL_OK;
}

int anl_nn_conv3d_bwd_data(const float* dz, const float* w, float* wt_work, float* dx, int cin, int cout, int D, int H,
                           int W, int ksize, int accumulate, anl_stream_t stream) {
    if (!dz || !w || !wt_work || !dx || cin < 1 || cout < 1 || (ksize != 1 && ksize != 3)) {
        set_error("anl_nn_conv3d_bwd_data: bad argument");
        return ANL_ERR_BADARG;
    }
    const int KK = ksize * ksize * ksize;
    cudaStream_t s = (cudaStream_t)stream;
    k_flip_weights<<<grid1((int64_t)cin * cout * KK), 256, 0, s>>>(w, wt_work, cin, cout, KK);
    ANL_LAUNCH_CHECK();
    // dx = conv(dz; w') with cout -> cin channels, no bias
    return anl_nn_conv3d(dz, wt_work, nullptr, dx, nullptr, cout, cin, D, H, W, ksize, 0, accumulate, stream);
}

int anl_nn_conv3d_bwd_weight(const float* x, const float* dz, float* part_work, int64_t part_floats, float* dw,
                             float* db, int cin, int cout, int D, int H, int W, int ksize, int accumulate,
                             anl_stream_t stream) {
    if (!x || !dz || !part_work || !dw || !db || cin < 1 || cout < 1 || (ksize != 1 && ksize != 3)) {
        set_error("anl_nn_conv3d_bwd_weight: bad argument");
        return ANL_ERR_BADARG;
    }
    const int KK = ksize * ksize * ksize;
    const int64_t vol = (int64_t)D * H * W;
    const int64_t per = (int64_t)cout * cin * KK + cout;  // floats per chunk (weights + bias)
    int nchunk = (int)std::min<int64_t>(64, std::max<int64_t>(1, vol / 2048));
    nchunk = (int)std::min<int64_t>(nchunk, part_floats / per);
    if (nchunk < 1) {
        set_error("anl_nn_conv3d_bwd_weight: workspace of %lld floats is below %lld", (long long)part_floats,
                  (long long)per);
        return ANL_ERR_BADARG;
    }
    const int64_t chunk = (vol + nchunk - 1) / nchunk;
    float* pw = part_work;
    float* pb = part_work + (int64_t)nchunk * cout * cin * KK;
    cudaStream_t s = (cudaStream_t)stream;
    dim3 grid(nchunk, cin, (cout + NN_CO - 1) / NN_CO);
    if (ksize == 3) k_conv3d_wgrad<3><<<grid, 512, 0, s>>>(x, dz, cin, cout, D, H, W, chunk, pw, pb);
    else k_conv3d_wgrad<1><<<grid, 512, 0, s>>>(x, dz, cin, cout, D, H, W, chunk, pw, pb);
    ANL_LAUNCH_CHECK();
    k_sum_parts<<<grid1((int64_t)cout * cin * KK), 256, 0, s>>>(pw, nchunk, (int64_t)cout * cin * KK, dw, accumulate);
    ANL_LAUNCH_CHECK();
    k_sum_parts<<<grid1(cout), 256, 0, s>>>(pb, nchunk, cout, db, accumulate);
    ANL_LAUNCH_CHECK();
    return ANL_OK;
}

int anl_nn_gelu_bwd(const float* z, const float* da, float* dz, int64_t n, anl_stream_t stream) {
    if (!z || !da || !dz || n < 0) {
        set_error("anl_nn_gelu_bwd: bad argument");
        return ANL_ERR_BADARG;
    }
    k_gelu_bwd<<<grid1(n), 256, 0, (cudaStream_t)stream>>>(n, z, da, dz);
    ANL_LAUNCH_CHECK();
    return ANL_OK;
}

int anl_nn_pool2(const float* x, float* y, int C, int D, int H, int W, int backward, int accumulate,
                 anl_stream_t stream) {
    if (!x || !y || C < 1 || D < 2 || H < 2 || W < 2 || (D | H | W) & 1) {
        set_error("anl_nn_pool2: bad argument (dims must be even)");
        return ANL_ERR_BADARG;
    }
    cudaStream_t s = (cudaStream_t)stream;
    if (backward) k_pool2_bwd<<<grid1((int64_t)C * D * H * W), 256, 0, s>>>(C, D, H, W, x, y, accumulate);
    else k_pool2<<<grid1((int64_t)C * D * H * W / 8), 256, 0, s>>>(C, D, H, W, x, y);
    ANL_LAUNCH_CHECK();
    return ANL_OK;
}

int anl_nn_up2(const float* x, float* y, int C, int D, int H, int W, int backward, anl_stream_t stream) {
    if (!x || !y || C < 1 || D < 2 || H < 2 || W < 2 || (D | H | W) & 1) {
        set_error("anl_nn_up2: bad argument (dims must be even)");
        return ANL_ERR_BADARG;
    }
    cudaStream_t s = (cudaStream_t)stream;
    if (backward) k_up2_bwd<<<grid1((int64_t)C * D * H * W / 8), 256, 0, s>>>(C, D, H, W, x, y);
    else k_up2<<<grid1((int64_t)C * D * H * W), 256, 0, s>>>(C, D, H, W, x, y);
    ANL_LAUNCH_CHECK();
    return ANL_OK;
}

int anl_nn_mse(const float* y, const float* tgt, const float* mask, float* dy, int C, int64_t vol, double* work,
               unsigned* counter, double* out2, anl_stream_t stream) {
    if (!y || !tgt || !mask || !dy || !work || !counter || !out2 || C < 1 || vol < 1) {
        set_error("anl_nn_mse: bad argument");
        return ANL_ERR_BADARG;
    }
    cudaStream_t s = (cudaStream_t)stream;
    const int nb = (int)std::min<int64_t>(kRedBlocks, (vol + NN_RT - 1) / NN_RT);
    k_mse<<<nb, NN_RT, 0, s>>>(C, vol, y, tgt, mask, dy, work, counter, out2);
    ANL_LAUNCH_CHECK();
    k_mse_grad<<<grid1((int64_t)C * vol), 256, 0, s>>>(C, vol, y, tgt, mask, out2, dy);
    ANL_LAUNCH_CHECK();
    return ANL_OK;
}

int anl_nn_adam(float* p, const float* g, float* m, float* v, int64_t n, double lr, double b1, double b2, double eps,
                int step, anl_stream_t stream) {
    if (!p || !g || !m || !v || n < 0 || step < 1) {
        set_error("anl_nn_adam: bad argument");
        return ANL_ERR_BADARG;
    }
    const float c1 = (float)(1.0 - std::pow(b1, step)), c2 = (float)(1.0 - std::pow(b2, step));
    k_adam<<<grid1(n), 256, 0, (cudaStream_t)stream>>>(n, p, g, m, v, (float)lr, (float)b1, (float)b2, (float)eps, c1,
                                                      c2);
    ANL_LAUNCH_CHECK();
    return ANL_OK;
}

}  // extern "C"
