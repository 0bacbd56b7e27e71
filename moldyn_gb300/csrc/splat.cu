// splat.cu -- headless particle render: the GUI viewer's sphere shading and
// bounding-box edges, ray-cast into an RGBA image instead of rasterised
// through wgpu (there is no graphics stack; the image is a plain buffer).
//
// Restates gui/src/visualizer/shader.wgsl:38-130 (instance colour by type or
// by speed gradient, Blinn-Phong-like shading 0.01 + max(n.l,0)^3 +
// max(n.h,0)^32 with l = -normalize(1,-1,1)), bounding_box.wgsl:26-59 (edge
// mask |p - 1/2| > 0.495 on two axes, alpha 0.1, blended), and the frame set-up
// of gui/src/visualizer/window.rs:940-990 (clear colour (0.01, 0.01, 0.02, 1),
// particles with depth test "less" and back faces culled, then the box with
// alpha blending, depth-tested but not depth-written).
//
// The GUI draws each particle as a 92-vertex icosphere; here the sphere is
// exact (a ray-cast impostor), so silhouettes are round rather than faceted.
// Every arithmetic step is an explicit round-to-nearest FP32 operation in a
// fixed order, so a CPU restatement with IEEE float32 reproduces the image
// bit for bit.  pow(x, 3) and pow(x, 32) are x*x*x and five squarings;
// normalize(v) is v / sqrt(v.v).
//
// Two passes: (1) one thread per particle walks the pixels of its sphere's
// conservative screen box (the projection of its view-space bounding cube,
// one pixel of margin) and keeps, per pixel, the smallest (depth, index) with
// one 64-bit atomicMin -- the nearest sphere, the lower index on equal depth,
// as the GUI's strict depth test over instances in order; (2) one thread per
// pixel shades its winner and blends the box edges in front of it.
#include <cuda_runtime.h>

#include <mutex>

#include <algorithm>
#include <vector>

#include "mdgb.h"

namespace {

struct SplatDev {
    float eye[3];
    float view[16];   // column-major, as the GUI's CameraUniform
    float p00, p11;   // projection scale factors (symmetric perspective)
    float znear, zfar;
    float gmin[4], gmid[4], gmax[4], grange[2];
    unsigned mode;
    float box[3];
    int draw_box;
    int width, height;
};

constexpr unsigned long long EMPTY = ~0ull;

// World-space direction of the ray through the centre of pixel (px, py): the
// view-space direction (x / P00, y / P11, -1) rotated back, so the ray
// parameter t is the view-space depth.
__device__ __forceinline__ void pixel_ray(const SplatDev& s, int px, int py, float d[3]) {
    const float xn = __fsub_rn(__fmul_rn(__fdiv_rn(__fadd_rn((float)px, 0.5f), (float)s.width), 2.0f), 1.0f);
    const float yn = __fsub_rn(1.0f, __fmul_rn(__fdiv_rn(__fadd_rn((float)py, 0.5f), (float)s.height), 2.0f));
    const float vx = __fdiv_rn(xn, s.p00), vy = __fdiv_rn(yn, s.p11);
#pragma unroll
    for (int j = 0; j < 3; ++j)
        d[j] = __fsub_rn(__fadd_rn(__fmul_rn(s.view[j * 4 + 0], vx), __fmul_rn(s.view[j * 4 + 1], vy)),
                         s.view[j * 4 + 2]);
}

__device__ __forceinline__ float dot3(const float a[3], const float b[3]) {
    return __fadd_rn(__fadd_rn(__fmul_rn(a[0], b[0]), __fmul_rn(a[1], b[1])), __fmul_rn(a[2], b[2]));
}

// Nearest intersection in front of the near plane, back faces culled (a ray
// starting inside the sphere sees nothing of it).
__device__ __forceinline__ bool hit_sphere(const SplatDev& s, const float d[3], const float c[3], float r,
                                           float& t) {
    const float oc[3] = {__fsub_rn(c[0], s.eye[0]), __fsub_rn(c[1], s.eye[1]), __fsub_rn(c[2], s.eye[2])};
    const float b = dot3(d, oc);
    const float a = dot3(d, d);
    const float cc = __fsub_rn(dot3(oc, oc), __fmul_rn(r, r));
    const float disc = __fsub_rn(__fmul_rn(b, b), __fmul_rn(a, cc));
    if (!(disc >= 0.0f)) return false;
    t = __fdiv_rn(__fsub_rn(b, __fsqrt_rn(disc)), a);
    return t >= s.znear && t <= s.zfar;
}

__device__ __forceinline__ void normalize3(float v[3]) {
    const float l = __fsqrt_rn(dot3(v, v));
    v[0] = __fdiv_rn(v[0], l);
    v[1] = __fdiv_rn(v[1], l);
    v[2] = __fdiv_rn(v[2], l);
}

// shader.wgsl:38-64 get_color and :86-113 the speed gradient
__device__ __forceinline__ void instance_color(const SplatDev& s, const float4 vel, const float4 mri, float col[3]) {
    col[0] = col[1] = col[2] = 0.0f;
    if (s.mode == 0u) {
        const unsigned id = (unsigned)mri.z;
        switch (id % 6u) {
            case 0u: col[0] = 1.0f; break;
            case 1u: col[1] = 1.0f; break;
            case 2u: col[2] = 1.0f; break;
            case 3u: col[0] = 1.0f; col[1] = 1.0f; break;
            case 4u: col[0] = 1.0f; col[2] = 1.0f; break;
            default: col[1] = 1.0f; col[2] = 1.0f; break;
        }
    } else if (s.mode == 1u) {
        const float v3[3] = {vel.x, vel.y, vel.z};
        const float gm = s.grange[0], gM = s.grange[1];
        float v = __fdiv_rn(__fsub_rn(__fsqrt_rn(dot3(v3, v3)), gm), __fsub_rn(gM, gm));
        if (gM <= gm) v = 1.0f;
        const float* lo = v < 0.5f ? s.gmin : s.gmid;
        const float* hi = v < 0.5f ? s.gmid : s.gmax;
        const float w = v < 0.5f ? __fmul_rn(v, 2.0f) : __fmul_rn(__fsub_rn(v, 0.5f), 2.0f);
        // mix(a, b, w) = a (1 - w) + b w
#pragma unroll
        for (int k = 0; k < 3; ++k) col[k] = __fadd_rn(__fmul_rn(lo[k], __fsub_rn(1.0f, w)), __fmul_rn(hi[k], w));
    }
}

__global__ void k_splat_depth(SplatDev s, const float4* __restrict__ part, long long n,
                              unsigned long long* __restrict__ depth) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 p = part[3 * i];
    const float r = part[3 * i + 2].y;
    const float c[3] = {p.x, p.y, p.z};
    // view-space centre: view * (c, 1)
    float cv[3];
#pragma unroll
    for (int j = 0; j < 3; ++j)
        cv[j] = s.view[12 + j] + s.view[j] * c[0] + s.view[4 + j] * c[1] + s.view[8 + j] * c[2];
    int x0 = 0, x1 = s.width - 1, y0 = 0, y1 = s.height - 1;
    const float rr = r * 1.001f + 1e-6f;
    if (cv[2] + rr < -s.znear) {
        // projection of the view-space bounding cube (its corners), one pixel of margin
        float xmin = 1e30f, xmax = -1e30f, ymin = 1e30f, ymax = -1e30f;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const float x = cv[0] + ((k & 1) ? rr : -rr), y = cv[1] + ((k & 2) ? rr : -rr);
            const float w = -(cv[2] + ((k & 4) ? rr : -rr));
            const float xn = s.p00 * x / w, yn = s.p11 * y / w;
            xmin = fminf(xmin, xn); xmax = fmaxf(xmax, xn);
            ymin = fminf(ymin, yn); ymax = fmaxf(ymax, yn);
        }
        if (xmax < -1.5f || xmin > 1.5f || ymax < -1.5f || ymin > 1.5f) return;   // off screen
        x0 = max(x0, (int)floorf((xmin + 1.0f) * 0.5f * s.width - 0.5f) - 1);
        x1 = min(x1, (int)ceilf((xmax + 1.0f) * 0.5f * s.width - 0.5f) + 1);
        y0 = max(y0, (int)floorf((1.0f - ymax) * 0.5f * s.height - 0.5f) - 1);
        y1 = min(y1, (int)ceilf((1.0f - ymin) * 0.5f * s.height - 0.5f) + 1);
    } else if (cv[2] - rr > -s.znear) {
        return;   // wholly behind the near plane
    }
    for (int py = y0; py <= y1; ++py) {
        for (int px = x0; px <= x1; ++px) {
            float d[3], t;
            pixel_ray(s, px, py, d);
            if (!hit_sphere(s, d, c, r, t)) continue;
            const unsigned long long key = ((unsigned long long)__float_as_uint(t) << 32) | (unsigned long long)i;
            atomicMin(depth + (size_t)py * s.width + px, key);
        }
    }
}

// bounding_box.wgsl:47-59 at a point on the box surface
__device__ __forceinline__ bool box_edge(const SplatDev& s, const float d[3], float t) {
    bool e[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float l = __fdiv_rn(__fadd_rn(s.eye[k], __fmul_rn(t, d[k])), s.box[k]);
        e[k] = fabsf(__fsub_rn(l, 0.5f)) > 0.495f;
    }
    return (e[0] && e[1]) || (e[0] && e[2]) || (e[1] && e[2]);
}

__global__ void k_splat_shade(SplatDev s, const float4* __restrict__ part, const unsigned long long* __restrict__ depth,
                              float4* __restrict__ out) {
    const int px = blockIdx.x * blockDim.x + threadIdx.x, py = blockIdx.y;
    if (px >= s.width) return;
    const size_t pix = (size_t)py * s.width + px;
    float rgb[3] = {0.01f, 0.01f, 0.02f};
    float d[3];
    pixel_ray(s, px, py, d);
    const unsigned long long key = depth[pix];
    float tz = s.zfar;
    if (key != EMPTY) {
        const long long i = (long long)(key & 0xffffffffull);
        const float4 p = part[3 * i], vel = part[3 * i + 1], mri = part[3 * i + 2];
        const float c[3] = {p.x, p.y, p.z};
        float t = 0.0f;
        hit_sphere(s, d, c, mri.y, t);
        tz = t;
        // shader.wgsl:121-130
        float nrm[3], pos[3], vv[3], h[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) nrm[k] = __fsub_rn(__fadd_rn(s.eye[k], __fmul_rn(t, d[k])), c[k]);
        normalize3(nrm);
#pragma unroll
        for (int k = 0; k < 3; ++k) pos[k] = __fadd_rn(c[k], __fmul_rn(nrm[k], mri.y));
#pragma unroll
        for (int k = 0; k < 3; ++k) vv[k] = __fsub_rn(s.eye[k], pos[k]);
        normalize3(vv);
        float l[3] = {1.0f, -1.0f, 1.0f};
        normalize3(l);
        l[0] = -l[0]; l[1] = -l[1]; l[2] = -l[2];
#pragma unroll
        for (int k = 0; k < 3; ++k) h[k] = __fadd_rn(vv[k], l[k]);
        normalize3(h);
        const float dl = fmaxf(dot3(nrm, l), 0.0f);
        float dh = fmaxf(dot3(nrm, h), 0.0f);
        const float p3 = __fmul_rn(__fmul_rn(dl, dl), dl);
#pragma unroll
        for (int k = 0; k < 5; ++k) dh = __fmul_rn(dh, dh);
        const float sh = __fadd_rn(__fadd_rn(0.01f, p3), dh);
        float col[3];
        instance_color(s, vel, mri, col);
#pragma unroll
        for (int k = 0; k < 3; ++k) rgb[k] = __fmul_rn(col[k], sh);
    }
    if (s.draw_box) {
        // slab test against [0, box]; the faces the ray crosses in front of
        // the nearest particle blend white at alpha 0.1 where they are edges
        float te = -1e30f, tx = 1e30f;
        bool ok = true;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            if (d[k] == 0.0f) {
                if (s.eye[k] < 0.0f || s.eye[k] > s.box[k]) ok = false;
                continue;
            }
            const float ta = __fdiv_rn(__fsub_rn(0.0f, s.eye[k]), d[k]);
            const float tb = __fdiv_rn(__fsub_rn(s.box[k], s.eye[k]), d[k]);
            te = fmaxf(te, fminf(ta, tb));
            tx = fminf(tx, fmaxf(ta, tb));
        }
        if (ok && te <= tx) {
            const float tf[2] = {te, tx};
#pragma unroll
            for (int f = 0; f < 2; ++f) {
                const float t = tf[f];
                if (t < s.znear || !(t < tz)) continue;
                if (!box_edge(s, d, t)) continue;
#pragma unroll
                for (int k = 0; k < 3; ++k) rgb[k] = __fadd_rn(0.1f, __fmul_rn(0.9f, rgb[k]));
            }
        }
    }
    out[pix] = make_float4(rgb[0], rgb[1], rgb[2], 1.0f);
}

}  // namespace

// Device buffers and a stream per GPU, kept between frames: they grow to the
// largest frame drawn and stay until the process exits.
namespace {
constexpr int SPLAT_MAX_DEVICES = 64;
struct SplatBuffers {
    void* part = nullptr;
    void* depth = nullptr;
    void* out = nullptr;
    size_t part_bytes = 0, depth_bytes = 0, out_bytes = 0;
    cudaStream_t st = nullptr;
};
SplatBuffers g_splat_buf[SPLAT_MAX_DEVICES];
std::mutex g_splat_mu[SPLAT_MAX_DEVICES];
}  // namespace

extern "C" MDGB_API int mdgb_splat(const float* particles, int64_t n, const mdgb_splat_params* prm, int width,
                                   int height, float* out_rgba) {
    if (n < 0 || (n > 0 && !particles) || !prm || !out_rgba || width <= 0 || height <= 0 ||
        n >= (int64_t)1 << 32 || (int64_t)width * height > ((int64_t)1 << 31))
        return MDGB_ERR_INVALID_ARGUMENT;
    SplatDev s{};
    for (int k = 0; k < 3; ++k) s.eye[k] = prm->view_pos[k];
    for (int k = 0; k < 16; ++k) s.view[k] = prm->view[k];
    s.p00 = prm->proj[0];
    s.p11 = prm->proj[5];
    // cgmath::perspective: proj[10] = (f+n)/(n-f), proj[14] = 2fn/(n-f)
    const float a = prm->proj[10], b = prm->proj[14];
    if (!(s.p00 != 0.0f && s.p11 != 0.0f && prm->proj[11] == -1.0f && a != 1.0f && a != -1.0f))
        return MDGB_ERR_INVALID_ARGUMENT;
    s.znear = b / (a - 1.0f);
    s.zfar = b / (a + 1.0f);
    for (int k = 0; k < 4; ++k) {
        s.gmin[k] = prm->gradient_min[k];
        s.gmid[k] = prm->gradient_mid[k];
        s.gmax[k] = prm->gradient_max[k];
    }
    s.grange[0] = prm->gradient_min_max[0];
    s.grange[1] = prm->gradient_min_max[1];
    s.mode = prm->mode;
    for (int k = 0; k < 3; ++k) s.box[k] = prm->box[k];
    s.draw_box = prm->draw_box && prm->box[0] > 0.0f && prm->box[1] > 0.0f && prm->box[2] > 0.0f;
    s.width = width;
    s.height = height;

    const size_t npix = (size_t)width * height;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= SPLAT_MAX_DEVICES) return MDGB_ERR_CUDA;
    // the device's buffers and stream, kept between frames (a frame of the
    // same or a smaller size allocates nothing); one frame at a time per device
    std::lock_guard<std::mutex> lock(g_splat_mu[dev]);
    SplatBuffers& B = g_splat_buf[dev];
    int rc = MDGB_OK;
    auto ok = [&](cudaError_t e) {
        if (e != cudaSuccess && rc == MDGB_OK) rc = MDGB_ERR_CUDA;
        return e == cudaSuccess;
    };
    auto grow = [&](void** p, size_t* have, size_t want) {
        if (*have >= want) return true;
        if (*p) cudaFree(*p);
        *p = nullptr;
        *have = 0;
        if (!ok(cudaMalloc(p, want))) return false;
        *have = want;
        return true;
    };
    const size_t part_bytes = std::max<size_t>(1, (size_t)n) * 3 * sizeof(float4);
    if ((B.st || ok(cudaStreamCreateWithFlags(&B.st, cudaStreamNonBlocking))) &&
        grow(&B.part, &B.part_bytes, part_bytes) && grow(&B.depth, &B.depth_bytes, npix * sizeof(unsigned long long)) &&
        grow(&B.out, &B.out_bytes, npix * sizeof(float4))) {
        cudaStream_t st = B.st;
        float4* d_part = static_cast<float4*>(B.part);
        unsigned long long* d_depth = static_cast<unsigned long long*>(B.depth);
        float4* d_out = static_cast<float4*>(B.out);
        if ((n == 0 || ok(cudaMemcpyAsync(d_part, particles, (size_t)n * 3 * sizeof(float4), cudaMemcpyHostToDevice, st))) &&
            ok(cudaMemsetAsync(d_depth, 0xff, npix * sizeof(unsigned long long), st))) {
            if (n > 0) k_splat_depth<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(s, d_part, n, d_depth);
            k_splat_shade<<<dim3((width + 127) / 128, height), 128, 0, st>>>(s, d_part, d_depth, d_out);
            if (ok(cudaGetLastError()) &&
                ok(cudaMemcpyAsync(out_rgba, d_out, npix * sizeof(float4), cudaMemcpyDeviceToHost, st)))
                ok(cudaStreamSynchronize(st));
        }
    }
    if (rc != MDGB_OK) cudaGetLastError();
    return rc;
}
