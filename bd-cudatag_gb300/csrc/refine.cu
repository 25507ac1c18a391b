// Photometric corner refinement (no counterpart in the reference; the
// reference's edge-line fit, gpu_detector.cu:881-1076, stays the default).
//
// For a quad with corners c (8 floats, TL TR BR BL) the homography H(c) of
// the reference's closed form (homography_from_unit_quad, :1249-1272) maps
// the unit square to the tag's black square.  The template is the tag's cell
// grid with a one-cell quiet zone: cells = dim + 2 per side (10 for
// tag36h11, 8 for tag16h5), each sampled at S x S sub-points.  Residual of
// sample s:
//     r_s = I(H(c)(u_s, v_s)) - (lo + (hi - lo) * t_s),   t_s in {0, 1}
// with I the frame sampled bilinearly by the reference's formula and out-of-
// frame samples masked (r_s = 0).  Loss = 0.5 * sum r_s^2 per quad.
//
// Derivatives: d(x, y)/dc comes from forward-mode duals through the closed
// form (8 derivative lanes); dI/d(x, y) is the bilinear patch gradient.  The
// adjoint kernel returns dL/dc and scatters dL/dI onto the four pixels of
// every sample.  The Gauss-Newton kernel builds J^T J and J^T r per quad,
// solves the damped 8x8 system in FP64 and iterates in shared memory.

#include <cuda_runtime.h>

#include <cstdint>

#include "bdcudatag/bdcudatag.h"
#include "bdcudatag/bdcudatag_gb300.h"
#include "families_data.inc"

namespace bdgb {
void set_last_error(const char* message);  // capi.cpp
}

namespace {

constexpr int kThreads = 256;

struct Dual {
    float v;
    float d[8];
};

__device__ __forceinline__ Dual dconst(float v) {
    Dual r;
    r.v = v;
#pragma unroll
    for (int k = 0; k < 8; ++k) r.d[k] = 0.0f;
    return r;
}

__device__ __forceinline__ Dual dvar(float v, int k) {
    Dual r = dconst(v);
    r.d[k] = 1.0f;
    return r;
}

__device__ __forceinline__ Dual operator+(const Dual& a, const Dual& b) {
    Dual r;
    r.v = a.v + b.v;
#pragma unroll
    for (int k = 0; k < 8; ++k) r.d[k] = a.d[k] + b.d[k];
    return r;
}

__device__ __forceinline__ Dual operator-(const Dual& a, const Dual& b) {
    Dual r;
    r.v = a.v - b.v;
#pragma unroll
    for (int k = 0; k < 8; ++k) r.d[k] = a.d[k] - b.d[k];
    return r;
}

__device__ __forceinline__ Dual operator*(const Dual& a, const Dual& b) {
    Dual r;
    r.v = a.v * b.v;
#pragma unroll
    for (int k = 0; k < 8; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
    return r;
}

__device__ __forceinline__ Dual operator/(const Dual& a, const Dual& b) {
    Dual r;
    r.v = a.v / b.v;
    const float inv2 = 1.0f / (b.v * b.v);
#pragma unroll
    for (int k = 0; k < 8; ++k) r.d[k] = (a.d[k] * b.v - a.v * b.d[k]) * inv2;
    return r;
}

// H and dH/dc (8 x 8) of the reference closed form, h[8] = 1.
__device__ bool homography_dual(const float* c, float h[8], float dh[8][8]) {
    const Dual x0 = dvar(c[0], 0), y0 = dvar(c[1], 1);
    const Dual x1 = dvar(c[2], 2), y1 = dvar(c[3], 3);
    const Dual x2 = dvar(c[4], 4), y2 = dvar(c[5], 5);
    const Dual x3 = dvar(c[6], 6), y3 = dvar(c[7], 7);
    const Dual dx1 = x1 - x2, dx2 = x3 - x2, dx3 = x0 - x1 + x2 - x3;
    const Dual dy1 = y1 - y2, dy2 = y3 - y2, dy3 = y0 - y1 + y2 - y3;
    const Dual det = dx1 * dy2 - dx2 * dy1;
    if (fabsf(det.v) < 1e-9f) return false;
    const Dual g = (dx3 * dy2 - dx2 * dy3) / det;
    const Dual k = (dx1 * dy3 - dx3 * dy1) / det;
    const Dual H[8] = {x1 - x0 + g * x1, x3 - x0 + k * x3, x0, y1 - y0 + g * y1,
                       y3 - y0 + k * y3, y0, g, k};
    for (int i = 0; i < 8; ++i) {
        h[i] = H[i].v;
        for (int j = 0; j < 8; ++j) dh[i][j] = H[i].d[j];
    }
    return true;
}

struct Sample {
    bool in;
    float val;    // frame value at the sample
    float r;      // residual
    float gx[8];  // d r / d c
    int64_t off;  // pixel offset of the top-left bilinear neighbour
    float w[4];   // bilinear weights (a, b, c, d)
};

struct QuadCtx {
    const uint8_t* image;
    int width, height;
    int64_t stride;
    float h[8];
    float dh[8][8];
    float lo, hi;
    const uint8_t* tmpl;
    int cells, spc;
};

// Sample s of the quad: position through H, bilinear value, gradient w.r.t.
// the corners.
__device__ __forceinline__ void eval_sample(const QuadCtx& q, int s, bool want_grad, Sample* out) {
    const int per_cell = q.spc * q.spc;
    const int cell = s / per_cell;
    const int sub = s - cell * per_cell;
    const int cy = cell / q.cells, cx = cell - cy * q.cells;
    const int sy = sub / q.spc, sx = sub - sy * q.spc;
    const float dim = static_cast<float>(q.cells - 2);
    const float u = (static_cast<float>(cx - 1) + (static_cast<float>(sx) + 0.5f) / q.spc) / dim;
    const float v = (static_cast<float>(cy - 1) + (static_cast<float>(sy) + 0.5f) / q.spc) / dim;
    const float nx = q.h[0] * u + q.h[1] * v + q.h[2];
    const float ny = q.h[3] * u + q.h[4] * v + q.h[5];
    const float den = q.h[6] * u + q.h[7] * v + 1.0f;
    const float x = nx / den, y = ny / den;
    out->in = den > 1e-6f && x >= 0.0f && y >= 0.0f && x < static_cast<float>(q.width - 1) &&
              y < static_cast<float>(q.height - 1);
    out->r = 0.0f;
    if (!out->in) return;
    const int ix = static_cast<int>(x), iy = static_cast<int>(y);
    const float fx = x - static_cast<float>(ix), fy = y - static_cast<float>(iy);
    out->off = static_cast<int64_t>(iy) * q.stride + ix;
    const uint8_t* p = q.image + out->off;
    const float a = p[0], b = p[1], c = p[q.stride], d = p[q.stride + 1];
    const float val = (a * (1.0f - fx) + b * fx) * (1.0f - fy) + (c * (1.0f - fx) + d * fx) * fy;
    out->val = val;
    const float t = q.tmpl[cell] ? 1.0f : 0.0f;
    out->r = val - (q.lo + (q.hi - q.lo) * t);
    out->w[0] = (1.0f - fx) * (1.0f - fy);
    out->w[1] = fx * (1.0f - fy);
    out->w[2] = (1.0f - fx) * fy;
    out->w[3] = fx * fy;
    if (!want_grad) return;
    const float Ix = (b - a) * (1.0f - fy) + (d - c) * fy;
    const float Iy = (c * (1.0f - fx) + d * fx) - (a * (1.0f - fx) + b * fx);
    const float inv = 1.0f / den;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const float dnx = q.dh[0][k] * u + q.dh[1][k] * v + q.dh[2][k];
        const float dny = q.dh[3][k] * u + q.dh[4][k] * v + q.dh[5][k];
        const float dden = q.dh[6][k] * u + q.dh[7][k] * v;
        const float dxk = (dnx - x * dden) * inv;
        const float dyk = (dny - y * dden) * inv;
        out->gx[k] = Ix * dxk + Iy * dyk;
    }
}

// Deterministic block sum of per-thread values (fixed tree).
template <int N>
__device__ void block_sum(float (&v)[N], float (*smem)[kThreads]) {
#pragma unroll
    for (int i = 0; i < N; ++i) smem[i][threadIdx.x] = v[i];
    __syncthreads();
    for (int off = kThreads / 2; off > 0; off >>= 1) {
        if (threadIdx.x < off) {
#pragma unroll
            for (int i = 0; i < N; ++i) smem[i][threadIdx.x] += smem[i][threadIdx.x + off];
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < N; ++i) v[i] = smem[i][0];
    __syncthreads();
}

__device__ bool load_quad(const bd_refine_args& a, int qi, const float* corners, QuadCtx* q) {
    q->image = a.images + static_cast<int64_t>(a.image_index ? a.image_index[qi] : 0) * a.image_pitch;
    q->width = a.width;
    q->height = a.height;
    q->stride = a.stride;
    q->cells = a.cells;
    q->spc = a.samples_per_cell;
    q->tmpl = a.templates + static_cast<int64_t>(qi) * a.cells * a.cells;
    q->lo = a.levels ? a.levels[2 * qi] : 0.0f;
    q->hi = a.levels ? a.levels[2 * qi + 1] : 255.0f;
    return homography_dual(corners, q->h, q->dh);
}

__global__ void __launch_bounds__(kThreads) k_refine_forward(bd_refine_args a, float* residuals,
                                                             float* loss) {
    __shared__ QuadCtx q;
    __shared__ int ok;
    __shared__ float red[1][kThreads];
    const int qi = blockIdx.x;
    if (threadIdx.x == 0) ok = load_quad(a, qi, a.corners + 8 * qi, &q) ? 1 : 0;
    __syncthreads();
    const int n = a.cells * a.cells * a.samples_per_cell * a.samples_per_cell;
    float acc[1] = {0.0f};
    for (int s = threadIdx.x; s < n; s += kThreads) {
        Sample smp;
        smp.r = 0.0f;
        if (ok) eval_sample(q, s, false, &smp);
        if (residuals) residuals[static_cast<int64_t>(qi) * n + s] = smp.r;
        acc[0] += 0.5f * smp.r * smp.r;
    }
    block_sum<1>(acc, red);
    if (threadIdx.x == 0 && loss) loss[qi] = acc[0];
}

__global__ void __launch_bounds__(kThreads) k_refine_backward(bd_refine_args a,
                                                              const float* grad_residuals,
                                                              float* grad_corners,
                                                              float* grad_images) {
    __shared__ QuadCtx q;
    __shared__ int ok;
    __shared__ float red[8][kThreads];
    const int qi = blockIdx.x;
    if (threadIdx.x == 0) ok = load_quad(a, qi, a.corners + 8 * qi, &q) ? 1 : 0;
    __syncthreads();
    const int n = a.cells * a.cells * a.samples_per_cell * a.samples_per_cell;
    float g[8] = {};
    float* gimg = grad_images
                      ? grad_images + static_cast<int64_t>(a.image_index ? a.image_index[qi] : 0) *
                                          (a.image_pitch)
                      : nullptr;
    for (int s = threadIdx.x; s < n && ok; s += kThreads) {
        Sample smp;
        eval_sample(q, s, true, &smp);
        if (!smp.in) continue;
        const float go = grad_residuals[static_cast<int64_t>(qi) * n + s];
#pragma unroll
        for (int k = 0; k < 8; ++k) g[k] += go * smp.gx[k];
        if (gimg) {
            float* p = gimg + smp.off;
            atomicAdd(p, go * smp.w[0]);
            atomicAdd(p + 1, go * smp.w[1]);
            atomicAdd(p + q.stride, go * smp.w[2]);
            atomicAdd(p + q.stride + 1, go * smp.w[3]);
        }
    }
    block_sum<8>(g, red);
    if (threadIdx.x < 8 && grad_corners) grad_corners[8 * qi + threadIdx.x] = g[threadIdx.x];
}

// Cholesky solve of (A + lambda * diag(A)) x = -b, 8 x 8, FP64.
__device__ bool solve8(const double A[8][8], const double b[8], double lambda, double x[8]) {
    double L[8][8] = {};
    for (int i = 0; i < 8; ++i) {
        for (int j = 0; j <= i; ++j) {
            double s = A[i][j] + (i == j ? lambda * A[i][i] : 0.0);
            for (int k = 0; k < j; ++k) s -= L[i][k] * L[j][k];
            if (i == j) {
                if (s <= 1e-12) return false;
                L[i][i] = sqrt(s);
            } else {
                L[i][j] = s / L[j][j];
            }
        }
    }
    double y[8];
    for (int i = 0; i < 8; ++i) {
        double s = -b[i];
        for (int k = 0; k < i; ++k) s -= L[i][k] * y[k];
        y[i] = s / L[i][i];
    }
    for (int i = 7; i >= 0; --i) {
        double s = y[i];
        for (int k = i + 1; k < 8; ++k) s -= L[k][i] * x[k];
        x[i] = s / L[i][i];
    }
    return true;
}

__global__ void __launch_bounds__(kThreads) k_refine_gauss_newton(bd_refine_args a, float* corners,
                                                                  int iterations, float* loss) {
    __shared__ QuadCtx q;
    __shared__ float c[8];
    __shared__ int ok;
    __shared__ float red[44][kThreads];
    const int qi = blockIdx.x;
    const int n = a.cells * a.cells * a.samples_per_cell * a.samples_per_cell;
    if (threadIdx.x < 8) c[threadIdx.x] = corners[8 * qi + threadIdx.x];
    __syncthreads();
    float last_loss = 0.0f;
    for (int it = 0; it <= iterations; ++it) {
        if (threadIdx.x == 0) ok = load_quad(a, qi, c, &q) ? 1 : 0;
        __syncthreads();
        if (!ok) break;
        // Photometric levels: mean intensity over black / white template cells.
        float lv[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        if (!a.levels) {
            for (int s = threadIdx.x; s < n; s += kThreads) {
                Sample smp;
                eval_sample(q, s, false, &smp);
                if (!smp.in) continue;
                const int cell = s / (a.samples_per_cell * a.samples_per_cell);
                lv[q.tmpl[cell] ? 2 : 0] += smp.val;
                lv[q.tmpl[cell] ? 3 : 1] += 1.0f;
            }
            block_sum<4>(lv, reinterpret_cast<float(*)[kThreads]>(red));
            if (threadIdx.x == 0) {
                q.lo = lv[1] > 0.0f ? lv[0] / lv[1] : 0.0f;
                q.hi = lv[3] > 0.0f ? lv[2] / lv[3] : 255.0f;
            }
            __syncthreads();
        }
        // Normal equations: 36 unique entries of J^T J, 8 of J^T r, loss.
        float acc[45] = {};
        for (int s = threadIdx.x; s < n; s += kThreads) {
            Sample smp;
            eval_sample(q, s, true, &smp);
            if (!smp.in) continue;
            int m = 0;
#pragma unroll
            for (int i = 0; i < 8; ++i) {
#pragma unroll
                for (int j = 0; j <= i; ++j) acc[m++] += smp.gx[i] * smp.gx[j];
            }
#pragma unroll
            for (int i = 0; i < 8; ++i) acc[36 + i] += smp.gx[i] * smp.r;
            acc[44] += 0.5f * smp.r * smp.r;
        }
        float part1[22], part2[23];
#pragma unroll
        for (int i = 0; i < 22; ++i) part1[i] = acc[i];
#pragma unroll
        for (int i = 0; i < 23; ++i) part2[i] = acc[22 + i];
        block_sum<22>(part1, red);
        block_sum<23>(part2, red);
        last_loss = part2[22];
        if (it == iterations) break;
        if (threadIdx.x == 0) {
            double A[8][8], b[8], x[8];
            int m = 0;
            for (int i = 0; i < 8; ++i) {
                for (int j = 0; j <= i; ++j) {
                    const float v = m < 22 ? part1[m] : part2[m - 22];
                    A[i][j] = A[j][i] = v;
                    ++m;
                }
            }
            for (int i = 0; i < 8; ++i) b[i] = part2[14 + i];
            if (solve8(A, b, 1e-4, x)) {
                for (int i = 0; i < 8; ++i) {
                    // Steps are clamped to 2 px per coordinate.
                    const double step = fmin(fmax(x[i], -2.0), 2.0);
                    c[i] = static_cast<float>(c[i] + step);
                }
            }
        }
        __syncthreads();
    }
    if (threadIdx.x < 8) corners[8 * qi + threadIdx.x] = c[threadIdx.x];
    if (threadIdx.x == 0 && loss) loss[qi] = last_loss;
}

int32_t check_args(const bd_refine_args* a) {
    if (!a || !a->images || !a->corners || !a->templates || a->count < 0 || a->cells < 3 ||
        a->cells > 16 || a->samples_per_cell < 1 || a->samples_per_cell > 16 || a->width < 2 ||
        a->height < 2 || a->stride < a->width || a->image_pitch < static_cast<int64_t>(a->stride) * a->height) {
        bdgb::set_last_error("bd_refine: invalid arguments");
        return BD_ERROR_INVALID_ARGUMENT;
    }
    return BD_OK;
}

int32_t launched() {
    const cudaError_t st = cudaGetLastError();
    if (st != cudaSuccess) {
        bdgb::set_last_error(cudaGetErrorString(st));
        return BD_ERROR_CUDA;
    }
    return BD_OK;
}

const uint64_t kCodes36[BD_CODEWORDS_36H11_COUNT] = {BD_CODEWORDS_36H11};
const uint64_t kCodes16[BD_CODEWORDS_16H5_COUNT] = {BD_CODEWORDS_16H5};

}  // namespace

extern "C" {

int32_t bd_tag_template(int32_t family, int32_t id, uint8_t* cells_out) {
    if (family < 0 || family > 1 || !cells_out) return BD_ERROR_INVALID_ARGUMENT;
    const int bits = family == 0 ? 6 : 4;
    const int count = family == 0 ? BD_CODEWORDS_36H11_COUNT : BD_CODEWORDS_16H5_COUNT;
    if (id < 0 || id >= count) return BD_ERROR_INVALID_ARGUMENT;
    const uint64_t code = family == 0 ? kCodes36[id] : kCodes16[id];
    const int cells = bits + 4;
    for (int cy = 0; cy < cells; ++cy) {
        for (int cx = 0; cx < cells; ++cx) {
            uint8_t v;
            if (cx == 0 || cy == 0 || cx == cells - 1 || cy == cells - 1) {
                v = 1;  // quiet zone
            } else if (cx == 1 || cy == 1 || cx == cells - 2 || cy == cells - 2) {
                v = 0;  // black border
            } else {
                const int pos = (cy - 2) * bits + (cx - 2);
                v = static_cast<uint8_t>((code >> (bits * bits - 1 - pos)) & 1ull);
            }
            cells_out[cy * cells + cx] = v;
        }
    }
    return cells;
}

int32_t bd_refine_forward(const bd_refine_args* args, float* residuals, float* loss,
                          void* cuda_stream) {
    const int32_t rc = check_args(args);
    if (rc != BD_OK) return rc;
    if (args->count == 0) return BD_OK;
    k_refine_forward<<<args->count, kThreads, 0, static_cast<cudaStream_t>(cuda_stream)>>>(
        *args, residuals, loss);
    return launched();
}

int32_t bd_refine_backward(const bd_refine_args* args, const float* grad_residuals,
                           float* grad_corners, float* grad_images, void* cuda_stream) {
    const int32_t rc = check_args(args);
    if (rc != BD_OK) return rc;
    if (!grad_residuals) {
        bdgb::set_last_error("bd_refine_backward: null residual gradient");
        return BD_ERROR_INVALID_ARGUMENT;
    }
    if (args->count == 0) return BD_OK;
    k_refine_backward<<<args->count, kThreads, 0, static_cast<cudaStream_t>(cuda_stream)>>>(
        *args, grad_residuals, grad_corners, grad_images);
    return launched();
}

int32_t bd_refine_gauss_newton(const bd_refine_args* args, float* corners_inout, int32_t iterations,
                               float* loss, void* cuda_stream) {
    const int32_t rc = check_args(args);
    if (rc != BD_OK) return rc;
    if (!corners_inout || iterations < 0 || iterations > 100) {
        bdgb::set_last_error("bd_refine_gauss_newton: bad corners or iteration count");
        return BD_ERROR_INVALID_ARGUMENT;
    }
    if (args->count == 0) return BD_OK;
    k_refine_gauss_newton<<<args->count, kThreads, 0, static_cast<cudaStream_t>(cuda_stream)>>>(
        *args, corners_inout, iterations, loss);
    return launched();
}

}  // extern "C"
