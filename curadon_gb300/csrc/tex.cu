// tex.cu -- projection kernels that filter through the texture unit.
//
// The texture unit interpolates with 9-bit fixed-point weights (8 fractional
// bits), the same hardware path the reference samples through
// (texture.hpp:81-87: linear filtering, border address mode, unnormalised
// coordinates), so these variants reproduce the reference's interpolation
// exactly; the launch shapes, the single launch over all views and the
// resident arrays are this project's.
//
//  k_fwd2d_tex    2D forward, tex2D on a 2D array refreshed per call
//  k_bwd2d_tex    2D backprojection, tex1DLayered on the sinogram rows
//  k_fwd3d_tex3   3D forward, tex3D (trilinear in the texture unit)
#include <algorithm>
#include <cfloat>
#include <cstring>
#include <vector>

#include "common.cuh"

namespace cg {

// ------------------------------------------------------------ objects

int make_texture(cudaArray_t arr, cudaTextureObject_t *tex) {
    cudaResourceDesc res;
    std::memset(&res, 0, sizeof(res));
    res.resType = cudaResourceTypeArray;
    res.res.array.array = arr;
    cudaTextureDesc td;
    std::memset(&td, 0, sizeof(td));
    td.addressMode[0] = td.addressMode[1] = td.addressMode[2] = cudaAddressModeBorder;
    td.filterMode = cudaFilterModeLinear;
    td.readMode = cudaReadModeElementType;
    td.normalizedCoords = 0;
    CG_TRY_CUDA(cudaCreateTextureObject(tex, &res, &td, nullptr));
    return CG_OK;
}

static int alloc_array(cudaArray_t *arr, size_t w, size_t h, size_t d, unsigned flags) {
    cudaChannelFormatDesc ch = cudaCreateChannelDesc<float>();
    CG_TRY_CUDA(cudaMalloc3DArray(arr, &ch, make_cudaExtent(w, h, d), flags));
    return CG_OK;
}

// Copies a dense (depth x height x width) float block into an array.
static int copy_to_array(cudaArray_t arr, const float *src, size_t w, size_t h, size_t d,
                         cudaStream_t s) {
    cudaMemcpy3DParms p;
    std::memset(&p, 0, sizeof(p));
    p.srcPtr = make_cudaPitchedPtr((void *)src, w * sizeof(float), w, h);
    p.dstArray = arr;
    p.extent = make_cudaExtent(w, h, d);
    p.kind = cudaMemcpyDeviceToDevice;
    CG_TRY_CUDA(cudaMemcpy3DAsync(&p, s));
    return CG_OK;
}

namespace {

// ------------------------------------------------------------ 2D forward

// Ray (u, view) of the reference's 2D forward (forward_2d.hpp:21-79) through
// the texture unit.
__device__ __forceinline__ void fwd2d_tex_ray(cudaTextureObject_t tex, float *__restrict__ sino,
                                              const float2 *__restrict__ tsrc,
                                              const float2 *__restrict__ tu0,
                                              const float2 *__restrict__ tdu, int W, int H,
                                              int det, float sx, float sy, int u, int view) {
    const float2 s = tsrc[view], o = tu0[view], du = tdu[view];
    const float fu = (float)u;
    const float dx = fmaf(du.x, fu, o.x);
    const float dy = fmaf(du.y, fu, o.y);
    float tmin = FLT_MIN, tmax = FLT_MAX;
    {
        const float t1 = __fdividef(-1.f - s.x, dx), t2 = __fdividef((float)W - s.x, dx);
        tmin = fminf(fmaxf(t1, tmin), fmaxf(t2, tmin));
        tmax = fmaxf(fminf(t1, tmax), fminf(t2, tmax));
    }
    {
        const float t1 = __fdividef(-1.f - s.y, dy), t2 = __fdividef((float)H - s.y, dy);
        tmin = fminf(fmaxf(t1, tmin), fmaxf(t2, tmin));
        tmax = fmaxf(fminf(t1, tmax), fminf(t2, tmax));
    }
    float *out = sino + (size_t)view * det + u;
    if ((double)tmin > (double)tmax - 1e-6) {
        *out = 0.f;
        return;
    }
    float x = fmaf(dx, tmin, s.x), y = fmaf(dy, tmin, s.y);
    const float tl = tmax - tmin;
    const float rdx = dx * tl, rdy = dy * tl;
    const float m = fmaxf(fabsf(rdx), fabsf(rdy));
    const int n = __float2int_rn(m);
    const float vx = rdx / m, vy = rdy / m;
    float acc = 0.f;
#pragma unroll 4
    for (int j = 0; j < n; ++j) {
        acc += tex2D<float>(tex, x, y);
        x += vx;
        y += vy;
    }
    *out = acc * hypotf(vx * sx, vy * sy);
}

__global__ void __launch_bounds__(256)
    k_fwd2d_tex(cudaTextureObject_t tex, float *__restrict__ sino,
                const float2 *__restrict__ tsrc, const float2 *__restrict__ tu0,
                const float2 *__restrict__ tdu, int W, int H, int det, int nangles, float sx,
                float sy) {
    const int u = blockIdx.x * blockDim.x + threadIdx.x;
    const int view = blockIdx.y * blockDim.y + threadIdx.y;
    if (u >= det || view >= nangles) return;
    fwd2d_tex_ray(tex, sino, tsrc, tu0, tdu, W, H, det, sx, sy, u, view);
}

// Many problems' texture forwards in one launch: blocks of 32 cells x 8
// views over a (problem, tile) work list, each problem with its own texture
// (bindless handles in the work list).
__global__ void __launch_bounds__(256)
    k_batch_fwd2d_tex(const Prob2d *__restrict__ probs, const int *__restrict__ start,
                      int count) {
    int lo = 0, hi = count - 1;
    const int b = blockIdx.x;
    while (lo < hi) {  // last problem whose first block is <= b
        const int mid = (lo + hi + 1) >> 1;
        if (start[mid] <= b) lo = mid; else hi = mid - 1;
    }
    const Prob2d &q = probs[lo];
    const int t = b - start[lo], tiles_u = (q.det + 31) / 32;
    const int u = (t % tiles_u) * 32 + threadIdx.x, view = (t / tiles_u) * 8 + threadIdx.y;
    if (u >= q.det || view >= q.nangles) return;
    fwd2d_tex_ray(q.tex, q.sino, q.src, q.u0, q.du, q.W, q.H, q.det, q.sx, q.sy, u, view);
}

// ------------------------------------------------------------ 2D backward

constexpr int kTexBwdRows = 4;
constexpr int kTexBwdViews = 256;

__global__ void __launch_bounds__(256)
    k_bwd2d_tex(float *__restrict__ vol, cudaTextureObject_t tex, const float4 *__restrict__ meta,
                int W, int H, int det, int v0, int nv, float sx, float sy, float ox, float oy,
                float ds, int ybase) {
    __shared__ float4 smeta[kTexBwdViews];
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    const int x = blockIdx.x * 32 + threadIdx.x;
    const int y0 = ybase + blockIdx.y * 32 + threadIdx.y;
    const float ex = (float)W / 2.0f, ey = (float)H / 2.0f, ed = (float)det / 2.0f;
    const float inv = __fdividef(1.0f, ds);
    const float X = ((float)x - ex) * sx + ox + 0.5f;
    const float SX = X * inv;
    float Y[kTexBwdRows], SY[kTexBwdRows], acc[kTexBwdRows];
#pragma unroll
    for (int r = 0; r < kTexBwdRows; ++r) {
        Y[r] = ((float)(y0 + 8 * r) - ey) * sy + oy + 0.5f;
        SY[r] = Y[r] * inv;
        acc[r] = 0.f;
    }
    for (int s0 = 0; s0 < nv; s0 += kTexBwdViews) {
        const int cnt = min(kTexBwdViews, nv - s0);
        __syncthreads();
        for (int i = tid; i < cnt; i += 256) smeta[i] = meta[v0 + s0 + i];
        __syncthreads();
#pragma unroll 4
        for (int j = 0; j < cnt; ++j) {
            const float4 m = smeta[j];
            const float layer = (float)(s0 + j);
#pragma unroll
            for (int r = 0; r < kTexBwdRows; ++r) {
                const float xi = m.x * X - m.y * Y[r];
                const float yi = m.y * SX + m.x * SY[r];
                const float w = __fdividef(m.z, xi + m.w);
                const float u = w * yi + ed;
                acc[r] = fmaf(tex1DLayered<float>(tex, u, (int)layer), w, acc[r]);
            }
        }
    }
    if (x < W) {
#pragma unroll
        for (int r = 0; r < kTexBwdRows; ++r) {
            const int y = y0 + 8 * r;
            if (y < H) vol[(size_t)y * W + x] += acc[r] * inv;
        }
    }
}

// ------------------------------------------------------------ 3D forward

struct RaySeg {
    float sx, sy, sz, dx, dy, dz, tmin, tmax, h;
    int nsteps;
    bool hit;
};

// Ray set-up of forward_3d.hpp:56-81 (intersection.h:12-28).
__device__ __forceinline__ RaySeg ray3d(const float4 o, const float4 du, const float4 dv,
                                        const float4 s, int iu, int iv, int X, int Y, int Z) {
    RaySeg r;
    const float fu = (float)iu, fv = (float)iv;
    const float detx = o.x + fu * du.x + fv * dv.x;
    const float dety = o.y + fu * du.y + fv * dv.y;
    const float detz = o.z + fu * du.z + fv * dv.z;
    r.sx = s.x, r.sy = s.y, r.sz = s.z;
    r.dx = detx - s.x, r.dy = dety - s.y, r.dz = detz - s.z;
    const float len = sqrtf(r.dx * r.dx + r.dy * r.dy + r.dz * r.dz);
    const long long nsamples = (long long)ceilf(__fdividef(len, 1.0f));
    float tmin = FLT_MIN, tmax = FLT_MAX;
    {
        const float t1 = __fdividef(-1.f - s.x, r.dx), t2 = __fdividef((float)(X + 1) - s.x, r.dx);
        tmin = fminf(fmaxf(t1, tmin), fmaxf(t2, tmin));
        tmax = fmaxf(fminf(t1, tmax), fminf(t2, tmax));
    }
    {
        const float t1 = __fdividef(-1.f - s.y, r.dy), t2 = __fdividef((float)(Y + 1) - s.y, r.dy);
        tmin = fminf(fmaxf(t1, tmin), fmaxf(t2, tmin));
        tmax = fmaxf(fminf(t1, tmax), fminf(t2, tmax));
    }
    {
        const float t1 = __fdividef(-1.f - s.z, r.dz), t2 = __fdividef((float)(Z + 1) - s.z, r.dz);
        tmin = fminf(fmaxf(t1, tmin), fmaxf(t2, tmin));
        tmax = fmaxf(fminf(t1, tmax), fminf(t2, tmax));
    }
    r.tmin = tmin, r.tmax = tmax;
    r.hit = tmin <= tmax;
    r.nsteps = r.hit ? (int)ceilf((tmax - tmin) * (float)nsamples) : 0;
    r.h = r.hit ? (tmax - tmin) / (float)r.nsteps : 0.f;
    if (!(r.h > 0.f) || !isfinite(tmax) || r.nsteps > (1 << 22)) r.hit = false;
    return r;
}

__global__ void __launch_bounds__(256)
    k_fwd3d_tex3(cudaTextureObject_t tex, float *__restrict__ sino,
                 const float4 *__restrict__ torg, const float4 *__restrict__ tdu,
                 const float4 *__restrict__ tdv, const float4 *__restrict__ tsrc, int X, int Y,
                 int Z, int U, int V, int P, bool exact_t) {
    const int iu = blockIdx.x * blockDim.x + threadIdx.x;
    const int iv = blockIdx.y * blockDim.y + threadIdx.y;
    const int view = blockIdx.z * blockDim.z + threadIdx.z;
    if (iu >= U || iv >= V || view >= P) return;
    const RaySeg r = ray3d(torg[view], tdu[view], tdv[view], tsrc[view], iu, iv, X, Y, Z);
    if (!r.hit) return;
    float acc = 0.f, t = r.tmin;
    for (int k = 0; k <= r.nsteps + 1; ++k) {
        if (!(t <= r.tmax)) break;
        acc += tex3D<float>(tex, fmaf(r.dx, t, r.sx) + 0.5f, fmaf(r.dy, t, r.sy) + 0.5f,
                            fmaf(r.dz, t, r.sz) + 0.5f);
        t = march_next(t, k, r.tmin, r.h, exact_t);
    }
    sino[((size_t)view * V + iv) * U + iu] = acc;
}

}  // namespace

// ------------------------------------------------------------ launchers

int launch_forward2d_tex(Plan2d &p, const float *vol, float *sino, cudaStream_t s) {
    if (!p.arr_vol) {
        int rc = alloc_array(&p.arr_vol, p.W, p.H, 0, cudaArrayDefault);
        if (rc) return rc;
        if ((rc = make_texture(p.arr_vol, &p.tex_vol))) return rc;
    }
    CG_TRY_CUDA(cudaMemcpy2DToArrayAsync(p.arr_vol, 0, 0, vol, sizeof(float) * p.W,
                                         sizeof(float) * p.W, p.H, cudaMemcpyDeviceToDevice, s));
    dim3 block(p.fwd_bx, p.fwd_by);
    dim3 grid(ceil_div(p.det, p.fwd_bx), ceil_div(p.nangles, p.fwd_by));
    if (grid.y > 65535) return set_error(CG_ERR_INVALID, "too many views for one launch");
    k_fwd2d_tex<<<grid, block, 0, s>>>(p.tex_vol, sino, p.d_src, p.d_u0, p.d_du, p.W, p.H, p.det,
                                       p.nangles, p.sx, p.sy);
    CG_TRY_CUDA(cudaGetLastError());
    return CG_OK;
}

int ensure_vol_texture(Plan2d &p) {
    if (!p.arr_vol) {
        int rc = alloc_array(&p.arr_vol, p.W, p.H, 0, cudaArrayDefault);
        if (rc) return rc;
        if ((rc = make_texture(p.arr_vol, &p.tex_vol))) return rc;
    }
    return CG_OK;
}

// Batched texture forward: each problem's volume into its plan's array, then
// one launch over the work list (stage-1 starts: 32 x 8 cell-view tiles).
int launch_batch2d_fwd_tex(const Prob2d *d_probs, const std::vector<Prob2d> &probs, int active,
                           const int *starts, int total, cudaStream_t s) {
    return launch_batch2d_fwd_tex_stage(d_probs, probs, active, starts, total, false, s);
}

int launch_batch2d_fwd_tex_stage(const Prob2d *d_probs, const std::vector<Prob2d> &probs,
                                 int active, const int *starts, int total, bool only_unchunked,
                                 cudaStream_t s) {
    for (int i = 0; i < active; ++i) {
        const Prob2d &q = probs[i];
        if (only_unchunked && q.chunked) continue;
        CG_TRY_CUDA(cudaMemcpy2DToArrayAsync(q.arr, 0, 0, q.vol, sizeof(float) * q.W,
                                             sizeof(float) * q.W, q.H, cudaMemcpyDeviceToDevice,
                                             s));
    }
    if (total == 0) return CG_OK;
    k_batch_fwd2d_tex<<<total, dim3(32, 8), 0, s>>>(d_probs, starts, (int)probs.size());
    CG_TRY_CUDA(cudaGetLastError());
    return CG_OK;
}

int launch_backward2d_tex(Plan2d &p, float *vol, const float *sino, cudaStream_t s) {
    constexpr int kLayers = 2048;  // layered 1D arrays hold at most 2048 layers
    if (!p.arr_sino) {
        const int layers = std::min(p.nangles, kLayers);
        int rc = alloc_array(&p.arr_sino, p.det, 0, layers, cudaArrayLayered);
        if (rc) return rc;
        if ((rc = make_texture(p.arr_sino, &p.tex_sino))) return rc;
    }
    dim3 grid(ceil_div(p.W, 32), ceil_div(p.H, 32));
    for (int v0 = 0; v0 < p.nangles; v0 += kLayers) {
        const int nv = std::min(kLayers, p.nangles - v0);
        int rc = copy_to_array(p.arr_sino, sino + (size_t)v0 * p.det, p.det, 1, nv, s);
        if (rc) return rc;
        k_bwd2d_tex<<<grid, dim3(32, 8), 0, s>>>(vol, p.tex_sino, p.d_bmeta, p.W, p.H, p.det, v0,
                                                 nv, p.sx, p.sy, p.ox, p.oy, p.ds, 0);
        CG_TRY_CUDA(cudaGetLastError());
    }
    return CG_OK;
}

int ensure_volume_texture3(Plan3d &p) {
    if (!p.arr3) {
        int rc = alloc_array(&p.arr3, p.X, p.Y, p.Z, cudaArrayDefault);
        if (rc) return rc;
        if ((rc = make_texture(p.arr3, &p.tex3))) return rc;
    }
    return CG_OK;
}

int upload_volume_texture3(Plan3d &p, const float *vol, cudaStream_t s) {
    if (int rc = ensure_volume_texture3(p)) return rc;
    return copy_to_array(p.arr3, vol, p.X, p.Y, p.Z, s);
}

int launch_forward3d_tex(Plan3d &p, const float *vol, float *sino, cudaStream_t s) {
    const dim3 block(p.fwd_bx, p.fwd_by, p.fwd_bz);
    const dim3 grid(ceil_div(p.U, p.fwd_bx), ceil_div(p.V, p.fwd_by), ceil_div(p.nangles, p.fwd_bz));
    if (grid.z > 65535) return set_error(CG_ERR_INVALID, "too many views for one launch");
    int rc = upload_volume_texture3(p, vol, s);
    if (rc) return rc;
    k_fwd3d_tex3<<<grid, block, 0, s>>>(p.tex3, sino, p.d_forg, p.d_fdu, p.d_fdv, p.d_fsrc, p.X,
                                        p.Y, p.Z, p.U, p.V, p.nangles, p.exact_t);
    CG_TRY_CUDA(cudaGetLastError());
    return CG_OK;
}

}  // namespace cg
