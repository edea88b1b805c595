// ps_nn_net.cu -- the learned warm start's network: a 4-level conv encoder-decoder (U-Net) in bf16
// with FP32 accumulation, trained and run entirely by this library's kernels.
//
// Layout: activations NHWC (channels contiguous), bf16. A 3x3 convolution ("same" padding) is
//   col  = im2col(x)                  [P][kpad]  (P = B*H*W, kpad = round_up(9*cin, 8), zero tail)
//   y    = relu(col * W^T + b)        tcgen05 GEMM, bias/ReLU/bf16 fused in the epilogue
// and its backward pass
//   dz   = dy * (y > 0)  (bf16; the bias gradient is summed in FP32 in the same kernel)
//   dW  += dz^T * col    (GEMM over K = P, split-K with FP32 atomics; col built transposed)
//   dcol = dz * W        (GEMM, B operand = W^T); dx = col2im(dcol) (gather, no atomics).
// Network (base 32 channels, input 2: log10 viscosity and rho*g; output 3: P, Vx, Vy at cells):
//   enc: [conv3 c->c, conv3 c->c] at 1, 1/4, 1/16, 1/64 resolution (c = 32, 64, 128, 256; 4x4 average
//        pooling between levels, so that the coarsest level's 3x3 convolutions span the whole
//        domain: 2-D Stokes flow is long-range); dec: nearest x4 upsampling, concatenation with the
//        encoder output of that level, [conv3, conv3] (256+128 -> 128, 128+64 -> 64, 64+32 -> 32);
//        1x1 conv 32 -> 3.
// Optimiser: Adam on FP32 master weights, bf16 copies (and transposes) refreshed after each step.
#include <cuda_bf16.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <random>
#include <vector>

#include "ps_common.cuh"
#include "ps_nn.cuh"

namespace ps {

typedef __nv_bfloat16 bf16;

// ---- kernels ------------------------------------------------------------------------------
static inline unsigned nblk(int64_t n, int t = 256) { return (unsigned)std::min<int64_t>((n + t - 1) / t, 1 << 20); }
#define GSTRIDE(i, n) for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (n); i += (int64_t)gridDim.x * blockDim.x)

// col[p][k] of a 3x3 "same" convolution over x [B][H][W][C], or (ldp > 0) colT[k][p] with row stride
// ldp >= P and zero columns P..ldp
__global__ void nn_im2col3_k(const bf16* __restrict__ x, int64_t P, int H, int W, int C, int kpad, bf16* col,
                             int64_t ldp) {
    const int64_t n = (ldp > 0 ? ldp : P) * kpad;
    GSTRIDE(i, n) {
        int64_t p, k;
        if (ldp > 0) {
            k = i / ldp;
            p = i - k * ldp;
        } else {
            p = i / kpad;
            k = i - p * kpad;
        }
        const int tap = (int)(k / C), c = (int)(k - (int64_t)tap * C);
        bf16 v = __float2bfloat16(0.0f);
        if (tap < 9 && p < P) {
            const int64_t b = p / ((int64_t)H * W);
            const int rem = (int)(p - b * H * W), y = rem / W, xx = rem - y * W;
            const int sy = y + tap / 3 - 1, sx = xx + tap % 3 - 1;
            if (sy >= 0 && sy < H && sx >= 0 && sx < W) v = x[((b * H + sy) * W + sx) * C + c];
        }
        col[i] = v;
    }
}

// dx[q][c] (+)= sum over the 3x3 taps of dcol[p(q, tap)][tap*C + c]
__global__ void nn_col2im3_k(const float* __restrict__ dcol, int64_t P, int H, int W, int C, int kpad, float* dx,
                             int accumulate) {
    const int64_t n = P * C;
    GSTRIDE(i, n) {
        const int64_t q = i / C;
        const int c = (int)(i - q * C);
        const int64_t b = q / ((int64_t)H * W);
        const int rem = (int)(q - b * H * W), y = rem / W, xx = rem - y * W;
        float s = 0.0f;
#pragma unroll
        for (int tap = 0; tap < 9; tap++) {
            const int oy = y - (tap / 3 - 1), ox = xx - (tap % 3 - 1);
            if (oy >= 0 && oy < H && ox >= 0 && ox < W)
                s += dcol[((b * H + oy) * W + ox) * (int64_t)kpad + (int64_t)tap * C + c];
        }
        dx[i] = accumulate ? dx[i] + s : s;
    }
}

// dz = dy * (y > 0) (relu) or dy, as bf16 [P][ldz] (zero columns C..ldz); gb[c] += sum_p dz (FP32)
__global__ void nn_relu_bwd_k(const float* __restrict__ dy, int ldy, const bf16* __restrict__ y, int64_t P, int C,
                              int relu, bf16* dz, int ldz, float* gb) {
    __shared__ float part[256];
    for (int c = threadIdx.x; c < 256; c += blockDim.x) part[c] = 0.0f;
    __syncthreads();
    const int64_t n = P * ldz;
    GSTRIDE(i, n) {
        const int64_t p = i / ldz;
        const int c = (int)(i - p * ldz);
        float v = 0.0f;
        if (c < C) {
            v = dy[p * ldy + c];
            if (relu && !(__bfloat162float(y[p * C + c]) > 0.0f)) v = 0.0f;
            atomicAdd(&part[c], v);
        }
        dz[i] = __float2bfloat16_rn(v);
    }
    __syncthreads();
    for (int c = threadIdx.x; c < C; c += blockDim.x) atomicAdd(gb + c, part[c]);
}

// out[c][r] = in[r][c] for a bf16 matrix [R][C] with row stride ld; out rows have stride ldo >= R
// with zero columns R..ldo (tiles of 32 x 32; the grid covers ldo)
__global__ void nn_transpose_k(const bf16* __restrict__ in, int64_t R, int C, int ld, bf16* out, int64_t ldo) {
    __shared__ bf16 t[32][33];
    const int64_t r0 = blockIdx.x * 32LL;
    const int c0 = blockIdx.y * 32;
    for (int j = threadIdx.y; j < 32; j += blockDim.y) {
        const int64_t r = r0 + j;
        const int c = c0 + threadIdx.x;
        t[j][threadIdx.x] = (r < R && c < C) ? in[r * ld + c] : __float2bfloat16(0.0f);
    }
    __syncthreads();
    for (int j = threadIdx.y; j < 32; j += blockDim.y) {
        const int c = c0 + j;
        const int64_t r = r0 + threadIdx.x;
        if (c < C && r < ldo) out[(int64_t)c * ldo + r] = t[threadIdx.x][j];
    }
}

// f x f average pooling of x [B][H][W][C] -> [B][H/f][W/f][C] (FP32 sum row by row, bf16 result)
__global__ void nn_pool_k(const bf16* __restrict__ x, int64_t B, int H, int W, int C, int f, bf16* y) {
    const int h = H / f, w = W / f;
    const int64_t n = B * h * w * C;
    const float inv = 1.0f / (float)(f * f);
    GSTRIDE(i, n) {
        const int c = (int)(i % C);
        const int64_t q = i / C;
        const int xx = (int)(q % w), yy = (int)((q / w) % h);
        const int64_t b = q / ((int64_t)w * h);
        const bf16* s = x + ((b * H + (int64_t)f * yy) * W + (int64_t)f * xx) * C + c;
        float v = 0.0f;
        for (int r = 0; r < f; r++)
            for (int k = 0; k < f; k++) v += __bfloat162float(s[((int64_t)r * W + k) * C]);
        y[i] = __float2bfloat16_rn(v * inv);
    }
}
// dx [B][H][W][C] (+)= dy [B][H/f][W/f][C] / f^2 broadcast
__global__ void nn_pool_bwd_k(const float* __restrict__ dy, int64_t B, int H, int W, int C, int f, float* dx,
                              int accumulate) {
    const int h = H / f, w = W / f;
    const int64_t n = B * H * W * C;
    const float inv = 1.0f / (float)(f * f);
    GSTRIDE(i, n) {
        const int c = (int)(i % C);
        const int64_t q = i / C;
        const int xx = (int)(q % W), yy = (int)((q / W) % H);
        const int64_t b = q / ((int64_t)W * H);
        const float v = inv * dy[((b * h + yy / f) * w + xx / f) * C + c];
        dx[i] = accumulate ? dx[i] + v : v;
    }
}
// y[b][Y][X][coff + c] = x[b][Y/f][X/f][c]   (x: [B][H/f][W/f][C], y row stride ldy)
__global__ void nn_up_k(const bf16* __restrict__ x, int64_t B, int H, int W, int C, int f, bf16* y, int ldy, int coff) {
    const int h = H / f, w = W / f;
    const int64_t n = B * H * W * C;
    GSTRIDE(i, n) {
        const int c = (int)(i % C);
        const int64_t q = i / C;
        const int xx = (int)(q % W), yy = (int)((q / W) % H);
        const int64_t b = q / ((int64_t)W * H);
        y[q * ldy + coff + c] = x[((b * h + yy / f) * w + xx / f) * C + c];
    }
}
// dx[b][y][x][c] = sum over the f x f children of dk[.][coff + c] (dk row stride ldk)
__global__ void nn_up_bwd_k(const float* __restrict__ dk, int ldk, int coff, int64_t B, int H, int W, int C, int f,
                            float* dx) {
    const int h = H / f, w = W / f;
    const int64_t n = B * h * w * C;
    GSTRIDE(i, n) {
        const int c = (int)(i % C);
        const int64_t q = i / C;
        const int xx = (int)(q % w), yy = (int)((q / w) % h);
        const int64_t b = q / ((int64_t)w * h);
        const int64_t p00 = (b * H + (int64_t)f * yy) * W + (int64_t)f * xx;
        float v = 0.0f;
        for (int r = 0; r < f; r++)
            for (int k = 0; k < f; k++) v += dk[(p00 + (int64_t)r * W + k) * ldk + coff + c];
        dx[i] = v;
    }
}
// dst[p][doff + c] = src[p][soff + c] (bf16 or FP32 copies of channel ranges)
template <typename T>
__global__ void nn_copy_ch_k(const T* __restrict__ src, int lds, int soff, int64_t P, int C, T* dst, int ldd, int doff) {
    const int64_t n = P * C;
    GSTRIDE(i, n) {
        const int64_t p = i / C;
        const int c = (int)(i - p * C);
        dst[p * ldd + doff + c] = src[p * lds + soff + c];
    }
}
__global__ void nn_f32_to_bf16_k(const float* __restrict__ a, int64_t n, bf16* b) {
    GSTRIDE(i, n) b[i] = __float2bfloat16_rn(a[i]);
}
// weighted mean squared error: loss += sum w (y - t)^2 * scale, dy = 2 w (y - t) * scale
__global__ void nn_mse_k(const float* __restrict__ y, const float* __restrict__ t, const float* __restrict__ w,
                         int64_t P, int C, float scale, float* dy, double* loss) {
    double s = 0.0;
    const int64_t n = P * C;
    GSTRIDE(i, n) {
        const float wi = w ? w[i / C] : 1.0f;
        const float d = y[i] - t[i];
        dy[i] = 2.0f * wi * d * scale;
        s += (double)(wi * d * d) * scale;
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xFFFFFFFFu, s, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, s);
}
// Adam on FP32 masters (Kingma & Ba): m, v moments; bias-corrected step; bf16 copy refreshed
__global__ void nn_adam_k(float* w, const float* __restrict__ g, float* m, float* v, int64_t n, float lr, float b1,
                          float b2, float eps, float c1, float c2, bf16* wb) {
    GSTRIDE(i, n) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.0f - b1) * gi;
        const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
        w[i] = wi;
        if (wb) wb[i] = __float2bfloat16_rn(wi);
    }
}
// dst [K][ldt] bf16 = src [N][K]^T (FP32 masters), zero columns N..ldt
__global__ void nn_wt_k(const float* __restrict__ src, int N, int K, bf16* dst, int ldt) {
    const int64_t n = (int64_t)K * ldt;
    GSTRIDE(i, n) {
        const int64_t k = i / ldt;
        const int c = (int)(i - k * ldt);
        dst[i] = __float2bfloat16_rn(c < N ? src[(int64_t)c * K + k] : 0.0f);
    }
}

// Bilinear sample of channel ch of an NHWC FP32 field (row stride W pixels) at (fy, fx), clamped to
// the exty x extx valid corner of the field.
__device__ __forceinline__ float nn_bilinear(const float* f, int W, int exty, int extx, int C, int ch, float fy,
                                             float fx) {
    fy = fminf(fmaxf(fy, 0.0f), (float)(exty - 1));
    fx = fminf(fmaxf(fx, 0.0f), (float)(extx - 1));
    const int y0 = min((int)fy, exty - 2), x0 = min((int)fx, extx - 2);
    const int y1 = y0 + 1, x1 = x0 + 1;
    const float ty = fy - y0, tx = fx - x0;
    const float a = f[((int64_t)y0 * W + x0) * C + ch], b = f[((int64_t)y0 * W + x1) * C + ch];
    const float c = f[((int64_t)y1 * W + x0) * C + ch], d = f[((int64_t)y1 * W + x1) * C + ch];
    return (1.0f - ty) * ((1.0f - tx) * a + tx * b) + ty * ((1.0f - tx) * c + tx * d);
}

// Network input at the network's grid (node (i, j) of an n x n node grid, replicated past n-1):
// log10(Mus) and Rog of the fine Stokes2D grid (nx x ny nodes, column-major) sampled bilinearly.
__global__ void nn_ws_input_k(const double* __restrict__ Mus, const double* __restrict__ Rog, int nx, int ny, int NH,
                              int NW, int nvalid, const float* sc, float* x) {
    const int64_t n = (int64_t)NH * NW;
    GSTRIDE(i, n) {
        const int row = (int)(i / NW), col = (int)(i - (int64_t)row * NW);  // row = y node, col = x node
        const float cx = (float)min(col, nvalid - 1) * (float)(nx - 1) / (float)(nvalid - 1);
        const float cy = (float)min(row, nvalid - 1) * (float)(ny - 1) / (float)(nvalid - 1);
        const int x0 = min((int)cx, nx - 2), y0 = min((int)cy, ny - 2);
        const float tx = cx - x0, ty = cy - y0;
        float lm = 0.0f, rg = 0.0f;
        const int xs[2] = {x0, x0 + 1}, ys[2] = {y0, y0 + 1};
        const float wx[2] = {1.0f - tx, tx}, wy[2] = {1.0f - ty, ty};
        for (int a = 0; a < 2; a++)
            for (int b = 0; b < 2; b++) {
                const int64_t o = xs[a] + (int64_t)nx * ys[b];
                lm += wx[a] * wy[b] * (float)log10(Mus[o]);
                rg += wx[a] * wy[b] * (float)Rog[o];
            }
        x[i * 2 + 0] = (lm - sc[0]) * sc[1];
        x[i * 2 + 1] = (rg - sc[2]) * sc[3];
    }
}
// Fine P (nx x ny), Vx ((nx+1) x ny), Vy (nx x (ny+1)) from the network output y [NH][NW][3], which
// holds the staggered arrays of an nvalid x nvalid node grid (P at (row iy, col ix) for nodes,
// Vx at (iy, face ix) with nvalid + 1 faces, Vy at (face iy, ix)), rescaled by sc[4..6]. Positions
// map through physical coordinates: node i at i*h, face i at (i - 1/2)*h.
__global__ void nn_ws_output_k(const float* __restrict__ y, int NH, int NW, int nvalid, int nx, int ny, const float* sc,
                               double* Pt, double* Vx, double* Vy) {
    const int64_t nP = (int64_t)nx * ny, nVx = (int64_t)(nx + 1) * ny, nVy = (int64_t)nx * (ny + 1);
    const float rx = (float)(nvalid - 1) / (float)(nx - 1), ry = (float)(nvalid - 1) / (float)(ny - 1);
    GSTRIDE(i, nP + nVx + nVy) {
        if (i < nP) {
            const int ix = (int)(i % nx), iy = (int)(i / nx);
            Pt[i] = (double)(nn_bilinear(y, NW, nvalid, nvalid, 3, 0, iy * ry, ix * rx) * sc[4]);
        } else if (i < nP + nVx) {
            const int64_t j = i - nP;
            const int ix = (int)(j % (nx + 1)), iy = (int)(j / (nx + 1));  // face between nodes ix-1 and ix
            // the wall faces carry no normal flow and the PT iteration never updates them
            Vx[j] = (ix == 0 || ix == nx)
                        ? 0.0
                        : (double)(nn_bilinear(y, NW, nvalid, nvalid + 1, 3, 1, iy * ry, (ix - 0.5f) * rx + 0.5f) * sc[5]);
        } else {
            const int64_t j = i - nP - nVx;
            const int ix = (int)(j % nx), iy = (int)(j / nx);
            Vy[j] = (iy == 0 || iy == ny)
                        ? 0.0
                        : (double)(nn_bilinear(y, NW, nvalid + 1, nvalid, 3, 2, (iy - 0.5f) * ry + 0.5f, ix * rx) * sc[6]);
        }
    }
}

// ---- network -------------------------------------------------------------------------------
struct Conv {
    int cin = 0, cout = 0, k = 3, relu = 1;
    int64_t kdim = 0, kpad = 0;
    int ldt = 0;         // row stride of the transposed bf16 weights
    float* Wf = nullptr;  // FP32 masters [cout][kpad]
    float* b = nullptr;
    float *gW = nullptr, *gb = nullptr, *mW = nullptr, *vW = nullptr, *mb = nullptr, *vb = nullptr;
    bf16* W = nullptr;   // bf16 copy [cout][kpad]
    bf16* Wt = nullptr;  // bf16 [kpad][ldt] = W^T
};

struct NNet {
    int H = 0, W = 0, Bmax = 0, base = 32;
    int pf = 4;  // pooling / upsampling factor between levels (levels at 1, 1/4, 1/16, 1/64)
    std::vector<Conv> conv;      // 15 layers, order below
    std::vector<void*> allocs;
    int64_t step = 0;
    float scales[8] = {0, 1, 0, 1, 1, 1, 1, 0};  // input offset/scale (2 channels), output scales (3)
    // activations (bf16) and their gradients (FP32)
    bf16 *x0, *a[15], *p1, *p2, *p3, *k2, *k1, *k0;
    float *y, *ga[15], *gp1, *gp2, *gp3, *gk2, *gk1, *gk0;
    // scratch
    bf16 *col, *colT, *dz, *dzT;
    float* dcol;
    double* loss;
    float* dsc;  // device copy of scales
    float *ws_x, *ws_y;
    int lastB = 0;
};

static int nn_alloc(NNet* n, void** p, size_t bytes) {
    cudaError_t e = cudaMalloc(p, std::max<size_t>(bytes, 256));
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(PS_ERR_NOMEM, "ps_nn: allocation of %zu bytes failed", bytes);
    }
    cudaMemset(*p, 0, std::max<size_t>(bytes, 256));
    n->allocs.push_back(*p);
    return PS_OK;
}
template <typename T>
static int nn_alloc_t(NNet* n, T** p, size_t count) {
    return nn_alloc(n, reinterpret_cast<void**>(p), count * sizeof(T));
}

static void nn_free(NNet* n) {
    for (void* p : n->allocs) cudaFree(p);
    n->allocs.clear();
}

// layer table: (cin, cout) in forward order
static void nn_layers(NNet* n) {
    const int c = n->base;
    const int spec[15][3] = {{2, c, 3},          {c, c, 3},          {c, 2 * c, 3},      {2 * c, 2 * c, 3},
                             {2 * c, 4 * c, 3},  {4 * c, 4 * c, 3},  {4 * c, 8 * c, 3},  {8 * c, 8 * c, 3},
                             {12 * c, 4 * c, 3}, {4 * c, 4 * c, 3},  {6 * c, 2 * c, 3},  {2 * c, 2 * c, 3},
                             {3 * c, c, 3},      {c, c, 3},          {c, 3, 1}};
    n->conv.resize(15);
    for (int i = 0; i < 15; i++) {
        Conv& L = n->conv[i];
        L.cin = spec[i][0];
        L.cout = spec[i][1];
        L.k = spec[i][2];
        L.relu = i < 14;
        L.kdim = (int64_t)L.k * L.k * L.cin;
        L.kpad = (L.kdim + 7) / 8 * 8;
        L.ldt = (L.cout + 7) / 8 * 8;
    }
}

static int nn_level_H(const NNet* n, int lev) {
    int h = n->H;
    for (int i = 0; i < lev; i++) h /= n->pf;
    return h;
}
static int nn_level_W(const NNet* n, int lev) {
    int w = n->W;
    for (int i = 0; i < lev; i++) w /= n->pf;
    return w;
}
static int64_t nn_level_P(const NNet* n, int B, int lev) { return (int64_t)B * nn_level_H(n, lev) * nn_level_W(n, lev); }

static int nn_refresh_bf16(NNet* n, Conv& L, cudaStream_t s) {
    const int64_t nw = (int64_t)L.cout * L.kpad;
    nn_f32_to_bf16_k<<<nblk(nw), 256, 0, s>>>(L.Wf, nw, L.W);
    nn_wt_k<<<nblk(L.kpad * L.ldt), 256, 0, s>>>(L.Wf, L.cout, (int)L.kpad, L.Wt, L.ldt);
    PS_CUDA_TRY(cudaGetLastError());
    return PS_OK;
}

static int nn_create(NNet* n, int H, int W, int Bmax, uint64_t seed) {
    n->H = H;
    n->W = W;
    n->Bmax = Bmax;
    nn_layers(n);
    std::mt19937_64 rng(seed);
    for (int i = 0; i < 15; i++) {
        Conv& L = n->conv[i];
        const size_t nw = (size_t)L.cout * L.kpad;
        PS_TRY(nn_alloc_t(n, &L.Wf, nw));
        PS_TRY(nn_alloc_t(n, &L.gW, nw));
        PS_TRY(nn_alloc_t(n, &L.mW, nw));
        PS_TRY(nn_alloc_t(n, &L.vW, nw));
        PS_TRY(nn_alloc_t(n, &L.b, L.cout));
        PS_TRY(nn_alloc_t(n, &L.gb, L.cout));
        PS_TRY(nn_alloc_t(n, &L.mb, L.cout));
        PS_TRY(nn_alloc_t(n, &L.vb, L.cout));
        PS_TRY(nn_alloc_t(n, &L.W, nw));
        PS_TRY(nn_alloc_t(n, &L.Wt, (size_t)L.kpad * L.ldt));
        // He initialisation of the kdim real columns; zero padding and biases
        std::normal_distribution<float> nd(0.0f, (float)std::sqrt((L.relu ? 2.0 : 0.1) / (double)L.kdim));
        std::vector<float> h(nw, 0.0f);
        for (int o = 0; o < L.cout; o++)
            for (int64_t k = 0; k < L.kdim; k++) h[(size_t)o * L.kpad + k] = nd(rng);
        PS_CUDA_TRY(cudaMemcpy(L.Wf, h.data(), nw * sizeof(float), cudaMemcpyHostToDevice));
        PS_TRY(nn_refresh_bf16(n, L, 0));
    }
    const int c = n->base;
    const int64_t P0 = nn_level_P(n, Bmax, 0), P1 = nn_level_P(n, Bmax, 1), P2 = nn_level_P(n, Bmax, 2),
                  P3 = nn_level_P(n, Bmax, 3);
    const int64_t Pl[15] = {P0, P0, P1, P1, P2, P2, P3, P3, P2, P2, P1, P1, P0, P0, P0};
    PS_TRY(nn_alloc_t(n, &n->x0, P0 * 2));
    for (int i = 0; i < 15; i++) {
        const int co = i == 14 ? 3 : n->conv[i].cout;
        if (i < 14) PS_TRY(nn_alloc_t(n, &n->a[i], Pl[i] * co));
        PS_TRY(nn_alloc_t(n, &n->ga[i], Pl[i] * co));
    }
    n->a[14] = nullptr;
    PS_TRY(nn_alloc_t(n, &n->y, P0 * 3));
    PS_TRY(nn_alloc_t(n, &n->p1, P1 * c));
    PS_TRY(nn_alloc_t(n, &n->p2, P2 * 2 * c));
    PS_TRY(nn_alloc_t(n, &n->p3, P3 * 4 * c));
    PS_TRY(nn_alloc_t(n, &n->k2, P2 * 12 * c));
    PS_TRY(nn_alloc_t(n, &n->k1, P1 * 6 * c));
    PS_TRY(nn_alloc_t(n, &n->k0, P0 * 3 * c));
    PS_TRY(nn_alloc_t(n, &n->gp1, P1 * c));
    PS_TRY(nn_alloc_t(n, &n->gp2, P2 * 2 * c));
    PS_TRY(nn_alloc_t(n, &n->gp3, P3 * 4 * c));
    PS_TRY(nn_alloc_t(n, &n->gk2, P2 * 12 * c));
    PS_TRY(nn_alloc_t(n, &n->gk1, P1 * 6 * c));
    PS_TRY(nn_alloc_t(n, &n->gk0, P0 * 3 * c));
    int64_t colmax = 0, dzmax = 0;
    for (int i = 0; i < 15; i++) {
        const int64_t Pk = (Pl[i] + 7) / 8 * 8;
        colmax = std::max(colmax, Pk * n->conv[i].kpad);
        dzmax = std::max(dzmax, Pk * (int64_t)n->conv[i].ldt);
    }
    PS_TRY(nn_alloc_t(n, &n->col, colmax));
    PS_TRY(nn_alloc_t(n, &n->colT, colmax));
    PS_TRY(nn_alloc_t(n, &n->dcol, colmax));
    PS_TRY(nn_alloc_t(n, &n->dz, dzmax));
    PS_TRY(nn_alloc_t(n, &n->dzT, dzmax));
    PS_TRY(nn_alloc_t(n, &n->loss, 1));
    PS_TRY(nn_alloc_t(n, &n->dsc, 8));
    PS_TRY(nn_alloc_t(n, &n->ws_x, (int64_t)H * W * 2));
    PS_TRY(nn_alloc_t(n, &n->ws_y, (int64_t)H * W * 3));
    PS_CUDA_TRY(cudaMemcpy(n->dsc, n->scales, sizeof(n->scales), cudaMemcpyHostToDevice));
    PS_CUDA_TRY(cudaDeviceSynchronize());
    return PS_OK;
}

// y = act(conv(x)); x [P][cin] bf16 at resolution (h, w); y bf16 [P][cout] (or FP32 for the last layer)
static int nn_conv_fwd(NNet* n, Conv& L, const bf16* x, int B, int h, int w, void* y, cudaStream_t s, int* err) {
    const int64_t P = (int64_t)B * h * w;
    GemmEpilogue e{};
    e.M = P;
    e.N = L.cout;
    e.ldc = L.cout;
    e.alpha = 1.0f;
    e.bias = L.b;
    e.relu = L.relu;
    e.out_bf16 = L.relu;  // hidden layers bf16, output layer FP32
    e.outh = static_cast<bf16*>(y);
    e.outf = static_cast<float*>(y);
    const bf16* A = x;
    if (L.k == 3) {
        nn_im2col3_k<<<nblk(P * L.kpad), 256, 0, s>>>(x, P, h, w, L.cin, (int)L.kpad, n->col, 0);
        A = n->col;
    }
    return nn_gemm(A, P, L.W, L.cout, L.kpad, e, 1, s, err);
}

// Backward of one layer: dy (FP32 [P][cout] with row stride ldy) -> gW, gb (accumulated) and,
// if dx is non-NULL, dx (FP32 [P][cin], overwritten or accumulated)
static int nn_conv_bwd(NNet* n, Conv& L, const bf16* x, const bf16* yact, const float* dy, int ldy, int B, int h, int w,
                       float* dx, int accumulate, cudaStream_t s, int* err) {
    const int64_t P = (int64_t)B * h * w;
    const int64_t Pk = (P + 7) / 8 * 8;  // pixel count padded for the weight-gradient GEMM's K (zeros)
    nn_relu_bwd_k<<<nblk(P * L.ldt), 256, 0, s>>>(dy, ldy, yact, P, L.cout, L.relu, n->dz, L.ldt, L.gb);
    // dz^T [cout][Pk]
    nn_transpose_k<<<dim3((unsigned)((Pk + 31) / 32), (unsigned)((L.cout + 31) / 32)), dim3(32, 8), 0, s>>>(
        n->dz, P, L.cout, L.ldt, n->dzT, Pk);
    const bf16* colT = nullptr;
    if (L.k == 3) {
        nn_im2col3_k<<<nblk(Pk * L.kpad), 256, 0, s>>>(x, P, h, w, L.cin, (int)L.kpad, n->colT, Pk);
        colT = n->colT;
    } else {
        nn_transpose_k<<<dim3((unsigned)((Pk + 31) / 32), (unsigned)((L.cin + 31) / 32)), dim3(32, 8), 0, s>>>(
            x, P, L.cin, L.cin, n->colT, Pk);
        colT = n->colT;
    }
    GemmEpilogue gw{};
    gw.M = L.cout;
    gw.N = L.kpad;
    gw.ldc = L.kpad;
    gw.alpha = 1.0f;
    gw.atomic = 1;
    gw.outf = L.gW;
    const int64_t kb = (Pk + 63) / 64;
    const int64_t tiles = ((L.cout + 127) / 128) * ((L.kpad + 127) / 128);
    const int split = (int)std::max<int64_t>(1, std::min<int64_t>(kb, (2 * 152 + tiles - 1) / tiles));
    PS_TRY(nn_gemm(n->dzT, L.cout, colT, L.kpad, Pk, gw, split, s, err));
    if (dx) {
        GemmEpilogue gd{};
        gd.M = P;
        gd.N = L.kpad;
        gd.ldc = L.kpad;
        gd.alpha = 1.0f;
        gd.outf = L.k == 3 ? n->dcol : (accumulate ? n->dcol : dx);
        PS_TRY(nn_gemm(n->dz, P, L.Wt, L.kpad, L.ldt, gd, 1, s, err));
        if (L.k == 3)
            nn_col2im3_k<<<nblk(P * L.cin), 256, 0, s>>>(n->dcol, P, h, w, L.cin, (int)L.kpad, dx, accumulate);
        else if (accumulate)
            return fail(PS_ERR_ARG, "1x1 layer gradient accumulation is not used");
    }
    PS_CUDA_TRY(cudaGetLastError());
    return PS_OK;
}

static int nn_forward(NNet* n, int B, cudaStream_t s, int* err) {
    const int c = n->base, f = n->pf;
    auto& L = n->conv;
    auto cv = [&](int i, const bf16* x, int lev, void* y) {
        return nn_conv_fwd(n, L[i], x, B, nn_level_H(n, lev), nn_level_W(n, lev), y, s, err);
    };
    auto pool = [&](const bf16* x, int lev, int C, bf16* y) {
        nn_pool_k<<<nblk(nn_level_P(n, B, lev + 1) * C), 256, 0, s>>>(x, B, nn_level_H(n, lev), nn_level_W(n, lev), C,
                                                                      f, y);
    };
    auto upcat = [&](const bf16* low, int Cl, const bf16* skip, int Cs, int lev, bf16* k) {
        const int64_t P = nn_level_P(n, B, lev);
        nn_up_k<<<nblk(P * Cl), 256, 0, s>>>(low, B, nn_level_H(n, lev), nn_level_W(n, lev), Cl, f, k, Cl + Cs, 0);
        nn_copy_ch_k<bf16><<<nblk(P * Cs), 256, 0, s>>>(skip, Cs, 0, P, Cs, k, Cl + Cs, Cl);
    };
    PS_TRY(cv(0, n->x0, 0, n->a[0]));
    PS_TRY(cv(1, n->a[0], 0, n->a[1]));
    pool(n->a[1], 0, c, n->p1);
    PS_TRY(cv(2, n->p1, 1, n->a[2]));
    PS_TRY(cv(3, n->a[2], 1, n->a[3]));
    pool(n->a[3], 1, 2 * c, n->p2);
    PS_TRY(cv(4, n->p2, 2, n->a[4]));
    PS_TRY(cv(5, n->a[4], 2, n->a[5]));
    pool(n->a[5], 2, 4 * c, n->p3);
    PS_TRY(cv(6, n->p3, 3, n->a[6]));
    PS_TRY(cv(7, n->a[6], 3, n->a[7]));
    upcat(n->a[7], 8 * c, n->a[5], 4 * c, 2, n->k2);
    PS_TRY(cv(8, n->k2, 2, n->a[8]));
    PS_TRY(cv(9, n->a[8], 2, n->a[9]));
    upcat(n->a[9], 4 * c, n->a[3], 2 * c, 1, n->k1);
    PS_TRY(cv(10, n->k1, 1, n->a[10]));
    PS_TRY(cv(11, n->a[10], 1, n->a[11]));
    upcat(n->a[11], 2 * c, n->a[1], c, 0, n->k0);
    PS_TRY(cv(12, n->k0, 0, n->a[12]));
    PS_TRY(cv(13, n->a[12], 0, n->a[13]));
    PS_TRY(cv(14, n->a[13], 0, n->y));
    PS_CUDA_TRY(cudaGetLastError());
    n->lastB = B;
    return PS_OK;
}

// dy: FP32 [P0][3] gradient of the output; accumulates gW, gb of every layer
static int nn_backward(NNet* n, const float* dy, cudaStream_t s, int* err) {
    const int B = n->lastB, c = n->base, f = n->pf;
    auto& L = n->conv;
    auto bw = [&](int i, const bf16* x, const bf16* yact, const float* g, int ldg, int lev, float* dx, int acc) {
        return nn_conv_bwd(n, L[i], x, yact, g, ldg, B, nn_level_H(n, lev), nn_level_W(n, lev), dx, acc, s, err);
    };
    auto catbwd = [&](const float* gk, int Cl, int Cs, int lev, float* glow, float* gskip) {
        const int64_t P = nn_level_P(n, B, lev), Pl = nn_level_P(n, B, lev + 1);
        nn_up_bwd_k<<<nblk(Pl * Cl), 256, 0, s>>>(gk, Cl + Cs, 0, B, nn_level_H(n, lev), nn_level_W(n, lev), Cl, f,
                                                  glow);
        nn_copy_ch_k<float><<<nblk(P * Cs), 256, 0, s>>>(gk, Cl + Cs, Cl, P, Cs, gskip, Cs, 0);
    };
    auto poolbwd = [&](const float* gp, int lev, int C, float* gx) {
        nn_pool_bwd_k<<<nblk(nn_level_P(n, B, lev) * C), 256, 0, s>>>(gp, B, nn_level_H(n, lev), nn_level_W(n, lev), C,
                                                                      f, gx, 1);
    };
    PS_TRY(bw(14, n->a[13], nullptr, dy, 3, 0, n->ga[13], 0));
    PS_TRY(bw(13, n->a[12], n->a[13], n->ga[13], c, 0, n->ga[12], 0));
    PS_TRY(bw(12, n->k0, n->a[12], n->ga[12], c, 0, n->gk0, 0));
    catbwd(n->gk0, 2 * c, c, 0, n->ga[11], n->ga[1]);
    PS_TRY(bw(11, n->a[10], n->a[11], n->ga[11], 2 * c, 1, n->ga[10], 0));
    PS_TRY(bw(10, n->k1, n->a[10], n->ga[10], 2 * c, 1, n->gk1, 0));
    catbwd(n->gk1, 4 * c, 2 * c, 1, n->ga[9], n->ga[3]);
    PS_TRY(bw(9, n->a[8], n->a[9], n->ga[9], 4 * c, 2, n->ga[8], 0));
    PS_TRY(bw(8, n->k2, n->a[8], n->ga[8], 4 * c, 2, n->gk2, 0));
    catbwd(n->gk2, 8 * c, 4 * c, 2, n->ga[7], n->ga[5]);
    PS_TRY(bw(7, n->a[6], n->a[7], n->ga[7], 8 * c, 3, n->ga[6], 0));
    PS_TRY(bw(6, n->p3, n->a[6], n->ga[6], 8 * c, 3, n->gp3, 0));
    poolbwd(n->gp3, 2, 4 * c, n->ga[5]);
    PS_TRY(bw(5, n->a[4], n->a[5], n->ga[5], 4 * c, 2, n->ga[4], 0));
    PS_TRY(bw(4, n->p2, n->a[4], n->ga[4], 4 * c, 2, n->gp2, 0));
    poolbwd(n->gp2, 1, 2 * c, n->ga[3]);
    PS_TRY(bw(3, n->a[2], n->a[3], n->ga[3], 2 * c, 1, n->ga[2], 0));
    PS_TRY(bw(2, n->p1, n->a[2], n->ga[2], 2 * c, 1, n->gp1, 0));
    poolbwd(n->gp1, 0, c, n->ga[1]);
    PS_TRY(bw(1, n->a[0], n->a[1], n->ga[1], c, 0, n->ga[0], 0));
    PS_TRY(bw(0, n->x0, n->a[0], n->ga[0], c, 0, nullptr, 0));
    PS_CUDA_TRY(cudaGetLastError());
    return PS_OK;
}

static int nn_zero_grad(NNet* n, cudaStream_t s) {
    for (auto& L : n->conv) {
        PS_CUDA_TRY(cudaMemsetAsync(L.gW, 0, (size_t)L.cout * L.kpad * sizeof(float), s));
        PS_CUDA_TRY(cudaMemsetAsync(L.gb, 0, (size_t)L.cout * sizeof(float), s));
    }
    return PS_OK;
}

static int nn_adam(NNet* n, float lr, float b1, float b2, float eps, cudaStream_t s) {
    n->step++;
    const float c1 = 1.0f - (float)std::pow((double)b1, (double)n->step);
    const float c2 = 1.0f - (float)std::pow((double)b2, (double)n->step);
    for (auto& L : n->conv) {
        const int64_t nw = (int64_t)L.cout * L.kpad;
        nn_adam_k<<<nblk(nw), 256, 0, s>>>(L.Wf, L.gW, L.mW, L.vW, nw, lr, b1, b2, eps, c1, c2, L.W);
        nn_adam_k<<<nblk(L.cout), 256, 0, s>>>(L.b, L.gb, L.mb, L.vb, L.cout, lr, b1, b2, eps, c1, c2, nullptr);
        nn_wt_k<<<nblk(L.kpad * L.ldt), 256, 0, s>>>(L.Wf, L.cout, (int)L.kpad, L.Wt, L.ldt);
    }
    PS_CUDA_TRY(cudaGetLastError());
    return PS_OK;
}

// parameters in the order layer by layer: W [cout][kdim] (the real columns), then b [cout]
static int64_t nn_param_count(const NNet* n) {
    int64_t t = 0;
    for (auto& L : n->conv) t += (int64_t)L.cout * L.kdim + L.cout;
    return t;
}
static int nn_copy_params(NNet* n, float* host, bool to_host, bool grads) {
    int64_t o = 0;
    for (auto& L : n->conv) {
        float* W = grads ? L.gW : L.Wf;
        float* b = grads ? L.gb : L.b;
        for (int r = 0; r < L.cout; r++) {
            float* dev = W + (int64_t)r * L.kpad;
            if (to_host)
                PS_CUDA_TRY(cudaMemcpy(host + o, dev, L.kdim * sizeof(float), cudaMemcpyDeviceToHost));
            else
                PS_CUDA_TRY(cudaMemcpy(dev, host + o, L.kdim * sizeof(float), cudaMemcpyHostToDevice));
            o += L.kdim;
        }
        if (to_host)
            PS_CUDA_TRY(cudaMemcpy(host + o, b, L.cout * sizeof(float), cudaMemcpyDeviceToHost));
        else
            PS_CUDA_TRY(cudaMemcpy(b, host + o, L.cout * sizeof(float), cudaMemcpyHostToDevice));
        o += L.cout;
    }
    if (!to_host && !grads)
        for (auto& L : n->conv) PS_TRY(nn_refresh_bf16(n, L, 0));
    PS_CUDA_TRY(cudaDeviceSynchronize());
    return PS_OK;
}

static NNet* as_net(void* p) { return static_cast<NNet*>(p); }

static int check_net(void* p, int B) {
    if (!p) return fail(PS_ERR_NULL, "ps_nn: NULL network");
    if (B < 1 || B > as_net(p)->Bmax) return fail(PS_ERR_ARG, "ps_nn: batch %d outside [1, %d]", B, as_net(p)->Bmax);
    return PS_OK;
}

}  // namespace ps

using namespace ps;

extern "C" {

int ps_nn_create(int64_t H, int64_t W, int32_t max_batch, uint64_t seed, void** net) {
    DeviceState* st = nullptr;
    PS_TRY(current_state(&st));
    if (!net) return fail(PS_ERR_NULL, "ps_nn_create: NULL output");
    *net = nullptr;
    if (H < 64 || W < 64 || H % 64 || W % 64 || H * W > (1 << 24))
        return fail(PS_ERR_SHAPE, "ps_nn_create: H, W must be multiples of 64 in [64, 4096]");
    if (max_batch < 1 || (int64_t)max_batch * H * W > ((int64_t)1 << 26))
        return fail(PS_ERR_ARG, "ps_nn_create: max_batch * H * W must be in [1, 2^26]");
    NNet* n = new NNet();
    int rc = nn_create(n, (int)H, (int)W, max_batch, seed);
    if (rc != PS_OK) {
        nn_free(n);
        delete n;
        return rc;
    }
    *net = n;
    return PS_OK;
}

int ps_nn_destroy(void* net) {
    if (!net) return PS_OK;
    cudaDeviceSynchronize();
    nn_free(as_net(net));
    delete as_net(net);
    return PS_OK;
}

int ps_nn_forward(void* net, const float* x, int32_t B, float* y, void* stream) {
    DeviceState* st = nullptr;
    PS_TRY(current_state(&st));
    PS_TRY(check_net(net, B));
    if (!x) return fail(PS_ERR_NULL, "ps_nn_forward: NULL input");
    NNet* n = as_net(net);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int64_t P0 = nn_level_P(n, B, 0);
    nn_f32_to_bf16_k<<<nblk(P0 * 2), 256, 0, s>>>(x, P0 * 2, n->x0);
    PS_TRY(nn_forward(n, B, s, st->d_err));
    if (y) PS_CUDA_TRY(cudaMemcpyAsync(y, n->y, P0 * 3 * sizeof(float), cudaMemcpyDeviceToDevice, s));
    return finish_launch(s, 1, "ps_nn_forward");
}

int ps_nn_zero_grad(void* net, void* stream) {
    PS_TRY(check_net(net, 1));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    PS_TRY(nn_zero_grad(as_net(net), s));
    return finish_launch(s, 1, "ps_nn_zero_grad");
}

int ps_nn_backward(void* net, const float* dy, void* stream) {
    DeviceState* st = nullptr;
    PS_TRY(current_state(&st));
    PS_TRY(check_net(net, 1));
    NNet* n = as_net(net);
    if (!dy) return fail(PS_ERR_NULL, "ps_nn_backward: NULL gradient");
    if (n->lastB < 1) return fail(PS_ERR_ARG, "ps_nn_backward: no forward pass to differentiate");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    PS_TRY(nn_backward(n, dy, s, st->d_err));
    return finish_launch(s, 1, "ps_nn_backward");
}

int ps_nn_adam_step(void* net, float lr, float beta1, float beta2, float eps, void* stream) {
    PS_TRY(check_net(net, 1));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    PS_TRY(nn_adam(as_net(net), lr, beta1, beta2, eps, s));
    return finish_launch(s, 1, "ps_nn_adam_step");
}

int ps_nn_train_step(void* net, const float* x, const float* t, const float* w, int32_t B, float lr, double* loss,
                     void* stream) {
    DeviceState* st = nullptr;
    PS_TRY(current_state(&st));
    PS_TRY(check_net(net, B));
    if (!x || !t) return fail(PS_ERR_NULL, "ps_nn_train_step: NULL input / target");
    NNet* n = as_net(net);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int64_t P0 = nn_level_P(n, B, 0);
    nn_f32_to_bf16_k<<<nblk(P0 * 2), 256, 0, s>>>(x, P0 * 2, n->x0);
    PS_TRY(nn_forward(n, B, s, st->d_err));
    PS_CUDA_TRY(cudaMemsetAsync(n->loss, 0, sizeof(double), s));
    nn_mse_k<<<nblk(P0 * 3), 256, 0, s>>>(n->y, t, w, P0, 3, 1.0f / (float)(P0 * 3), n->ga[14], n->loss);
    PS_TRY(nn_zero_grad(n, s));
    PS_TRY(nn_backward(n, n->ga[14], s, st->d_err));
    PS_TRY(nn_adam(n, lr, 0.9f, 0.999f, 1e-8f, s));
    if (loss) {
        PS_CUDA_TRY(cudaMemcpyAsync(loss, n->loss, sizeof(double), cudaMemcpyDeviceToHost, s));
    }
    return finish_launch(s, 1, "ps_nn_train_step");
}

int ps_nn_get_activation(void* net, int32_t layer, float* host) {
    PS_TRY(check_net(net, 1));
    NNet* n = as_net(net);
    if (!host) return fail(PS_ERR_NULL, "NULL buffer");
    if (layer < 0 || layer > 14 || n->lastB < 1) return fail(PS_ERR_ARG, "ps_nn_get_activation: no layer %d output", layer);
    static const int lev[15] = {0, 0, 1, 1, 2, 2, 3, 3, 2, 2, 1, 1, 0, 0, 0};
    const int64_t cnt = nn_level_P(n, n->lastB, lev[layer]) * (layer == 14 ? 3 : n->conv[layer].cout);
    if (layer == 14) {
        PS_CUDA_TRY(cudaMemcpy(host, n->y, cnt * sizeof(float), cudaMemcpyDeviceToHost));
        return PS_OK;
    }
    std::vector<bf16> h(cnt);
    PS_CUDA_TRY(cudaMemcpy(h.data(), n->a[layer], cnt * sizeof(bf16), cudaMemcpyDeviceToHost));
    for (int64_t i = 0; i < cnt; i++) host[i] = __bfloat162float(h[i]);
    return PS_OK;
}

int ps_nn_param_count(void* net, int64_t* count) {
    PS_TRY(check_net(net, 1));
    if (!count) return fail(PS_ERR_NULL, "NULL output");
    *count = nn_param_count(as_net(net));
    return PS_OK;
}
int ps_nn_get_params(void* net, float* host) {
    PS_TRY(check_net(net, 1));
    if (!host) return fail(PS_ERR_NULL, "NULL buffer");
    return nn_copy_params(as_net(net), host, true, false);
}
int ps_nn_set_params(void* net, const float* host) {
    PS_TRY(check_net(net, 1));
    if (!host) return fail(PS_ERR_NULL, "NULL buffer");
    return nn_copy_params(as_net(net), const_cast<float*>(host), false, false);
}
int ps_nn_get_grads(void* net, float* host) {
    PS_TRY(check_net(net, 1));
    if (!host) return fail(PS_ERR_NULL, "NULL buffer");
    return nn_copy_params(as_net(net), host, true, true);
}
int ps_nn_set_scales(void* net, const float scales[8]) {
    PS_TRY(check_net(net, 1));
    if (!scales) return fail(PS_ERR_NULL, "NULL scales");
    memcpy(as_net(net)->scales, scales, sizeof(float) * 8);
    PS_CUDA_TRY(cudaMemcpy(as_net(net)->dsc, scales, sizeof(float) * 8, cudaMemcpyHostToDevice));
    return PS_OK;
}
int ps_nn_get_scales(void* net, float scales[8]) {
    PS_TRY(check_net(net, 1));
    if (!scales) return fail(PS_ERR_NULL, "NULL scales");
    memcpy(scales, as_net(net)->scales, sizeof(float) * 8);
    return PS_OK;
}

// File: "PSNN" magic, version 1, H, W, base, 8 scales, then per layer W [cout][kdim] bf16 and b
// [cout] FP32 (what inference uses; training resumes from the bf16 weights).
int ps_nn_save(void* net, const char* path) {
    PS_TRY(check_net(net, 1));
    if (!path) return fail(PS_ERR_NULL, "NULL path");
    NNet* n = as_net(net);
    std::vector<float> p(nn_param_count(n));
    PS_TRY(nn_copy_params(n, p.data(), true, false));
    FILE* fh = fopen(path, "wb");
    if (!fh) return fail(PS_ERR_ARG, "ps_nn_save: cannot open %s", path);
    const int32_t hdr[5] = {0x4E4E5350, 1, n->H, n->W, n->base};
    bool ok = fwrite(hdr, sizeof(hdr), 1, fh) == 1 && fwrite(n->scales, sizeof(n->scales), 1, fh) == 1;
    int64_t o = 0;
    for (auto& L : n->conv) {
        std::vector<__nv_bfloat16> wb((size_t)L.cout * L.kdim);
        for (size_t i = 0; i < wb.size(); i++) wb[i] = __float2bfloat16_rn(p[o + i]);
        o += (int64_t)wb.size();
        ok = ok && fwrite(wb.data(), sizeof(wb[0]), wb.size(), fh) == wb.size();
        ok = ok && fwrite(p.data() + o, sizeof(float), L.cout, fh) == (size_t)L.cout;
        o += L.cout;
    }
    fclose(fh);
    return ok ? PS_OK : fail(PS_ERR_ARG, "ps_nn_save: write to %s failed", path);
}

int ps_nn_load(void* net, const char* path) {
    PS_TRY(check_net(net, 1));
    if (!path) return fail(PS_ERR_NULL, "NULL path");
    NNet* n = as_net(net);
    FILE* fh = fopen(path, "rb");
    if (!fh) return fail(PS_ERR_ARG, "ps_nn_load: cannot open %s", path);
    int32_t hdr[5];
    float sc[8];
    bool ok = fread(hdr, sizeof(hdr), 1, fh) == 1 && fread(sc, sizeof(sc), 1, fh) == 1 && hdr[0] == 0x4E4E5350 &&
              hdr[1] == 1 && hdr[4] == n->base;
    std::vector<float> p(nn_param_count(n));
    int64_t o = 0;
    for (auto& L : n->conv) {
        if (!ok) break;
        std::vector<__nv_bfloat16> wb((size_t)L.cout * L.kdim);
        ok = fread(wb.data(), sizeof(wb[0]), wb.size(), fh) == wb.size();
        for (size_t i = 0; i < wb.size(); i++) p[o + i] = __bfloat162float(wb[i]);
        o += (int64_t)wb.size();
        ok = ok && fread(p.data() + o, sizeof(float), L.cout, fh) == (size_t)L.cout;
        o += L.cout;
    }
    fclose(fh);
    if (!ok) return fail(PS_ERR_ARG, "ps_nn_load: %s is not a weight file of this network", path);
    PS_TRY(nn_copy_params(n, p.data(), false, false));
    return ps_nn_set_scales(net, sc);
}

// Warm start of the Stokes2D PT solver: the network's prediction of P, Vx, Vy for the viscosity
// and buoyancy of f (sampled onto the network's node grid), interpolated onto f's staggered
// arrays; dVxdtau and dVydtau are zeroed (FP64 fields).
int ps_stokes2d_warm_start(void* net, const ps_stokes2d_fields* f, int32_t nvalid, void* stream) {
    DeviceState* st = nullptr;
    PS_TRY(current_state(&st));
    PS_TRY(check_net(net, 1));
    if (!f) return fail(PS_ERR_NULL, "NULL fields");
    NNet* n = as_net(net);
    const int64_t nx = f->Pt.n[0], ny = f->Pt.n[1];
    if (f->Pt.dtype != PS_F64 || f->Mus.dtype != PS_F64 || nx < 3 || ny < 3)
        return fail(PS_ERR_DTYPE, "ps_stokes2d_warm_start: FP64 fields with nx, ny >= 3 required");
    if (f->Vx.n[0] != nx + 1 || f->Vy.n[1] != ny + 1 || f->Mus.n[0] != nx || f->Rog.n[1] != ny)
        return fail(PS_ERR_SHAPE, "ps_stokes2d_warm_start: incoherent field sizes");
    if (nvalid < 2 || nvalid >= n->H || nvalid >= n->W) return fail(PS_ERR_ARG, "ps_stokes2d_warm_start: bad nvalid");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int64_t P0 = (int64_t)n->H * n->W;
    nn_ws_input_k<<<nblk(P0), 256, 0, s>>>(static_cast<const double*>(f->Mus.ptr), static_cast<const double*>(f->Rog.ptr),
                                           (int)nx, (int)ny, n->H, n->W, nvalid, n->dsc, n->ws_x);
    nn_f32_to_bf16_k<<<nblk(P0 * 2), 256, 0, s>>>(n->ws_x, P0 * 2, n->x0);
    PS_TRY(nn_forward(n, 1, s, st->d_err));
    const int64_t tot = nx * ny + (nx + 1) * ny + nx * (ny + 1);
    nn_ws_output_k<<<nblk(tot), 256, 0, s>>>(n->y, n->H, n->W, nvalid, (int)nx, (int)ny, n->dsc,
                                             static_cast<double*>(f->Pt.ptr), static_cast<double*>(f->Vx.ptr),
                                             static_cast<double*>(f->Vy.ptr));
    PS_CUDA_TRY(cudaMemsetAsync(f->dVxdtau.ptr, 0, (size_t)numel(f->dVxdtau) * 8, s));
    PS_CUDA_TRY(cudaMemsetAsync(f->dVydtau.ptr, 0, (size_t)numel(f->dVydtau) * 8, s));
    // the loop body's free-slip copies, so the start state satisfies them like every PT iterate
    PS_TRY(ps_bc_y2d(f->Vx, stream, 0));
    PS_TRY(ps_bc_x2d(f->Vy, stream, 0));
    return finish_launch(s, 1, "ps_stokes2d_warm_start");
}

}  // extern "C"
