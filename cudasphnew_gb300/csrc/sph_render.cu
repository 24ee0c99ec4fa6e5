// Headless particle renderer: the sphere-imposter splatting of the
// reference's TwoScaleStateSub renderer (twoscalestatesub.cpp:84-161 and its
// shaders twoscalestatesub_{v,g,f}.glsl) as two CUDA passes into a device
// image, no graphics API.
//
// What the shaders compute, per particle p of world radius R:
//   eye  = view * (p, 1)                                  (vertex shader)
//   c    = proj * eye / -eye.z        (the quad's centre, w = 1 after the division)
//   d    = (proj[0][0], proj[1][1]) * R / -eye.z          (half extents)
//   quad = c +- d, relCoord = +-1 at its corners          (geometry shader)
//   per fragment: (u, v) = relCoord, discard when u^2 + v^2 > 1,
//   n = (u, v, sqrt(1 - u^2 - v^2)), zEye = eye.z + R n.z,
//   depth = -proj[2][2] - proj[2][3] / zEye,
//   colour = (0.9 + 0.1 max(0, n.z)) * (particleColor, 1)  (fragment shader)
// with column-major matrices (proj[c][r] = m[4c + r]).  The quad has w = 1,
// so relCoord interpolates linearly in screen space: at a pixel centre it is
// ((x - c.x) / d.x, (y - c.y) / d.y) in normalised device coordinates.
//
// Rasterisation: GL covers a pixel whose centre lies inside the quad; the
// depth test is GL_LESS against a depth buffer cleared to 1, depth clamped
// to [0, 1] and stored as 24-bit fixed point; among equal stored depths the
// fragment drawn first stays.  The splat pass takes, per pixel, the minimum
// of (24-bit depth << 32 | draw index) with a 64-bit atomicMin, which is that
// rule exactly (the draw index orders the passes and their particles as the
// reference draws them).  The shade pass recomputes the winning fragment's
// colour.  The clear colour is white; the image is RGBA8, rows top to bottom.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <vector>

#include "sph_device.cuh"
#include "sph_sim.h"

namespace sph {
namespace {

constexpr unsigned long long EMPTY_KEY = ~0ull;

struct Camera {
    float v[16], p[16];  // column-major
};

// One draw call: `count` particles ids[k] (or k) of `pos`, radius, colour.
struct Pass {
    const float4* pos;
    const int* ids;
    int count;
    int base;  // draw index of its first particle
    float radius;
    float rgb[3];
};

struct Passes {
    Pass p[3];
    int num;
};

struct Frag {
    float cx, cy, dx, dy, ez;
    bool ok;
};

// Vertex + geometry shader of one particle: the quad in NDC and the eye depth.
__device__ __forceinline__ Frag project(const Camera& c, float4 x, float R) {
    Frag f;
    const float ex = c.v[0] * x.x + c.v[4] * x.y + c.v[8] * x.z + c.v[12];
    const float ey = c.v[1] * x.x + c.v[5] * x.y + c.v[9] * x.z + c.v[13];
    const float ez = c.v[2] * x.x + c.v[6] * x.y + c.v[10] * x.z + c.v[14];
    const float ew = c.v[3] * x.x + c.v[7] * x.y + c.v[11] * x.z + c.v[15];
    const float w = -ez;
    const float px = c.p[0] * ex + c.p[4] * ey + c.p[8] * ez + c.p[12] * ew;
    const float py = c.p[1] * ex + c.p[5] * ey + c.p[9] * ez + c.p[13] * ew;
    const float pz = c.p[2] * ex + c.p[6] * ey + c.p[10] * ez + c.p[14] * ew;
    f.cx = px / w;
    f.cy = py / w;
    f.dx = c.p[0] * R / w;
    f.dy = c.p[5] * R / w;
    f.ez = ez;
    // behind the eye, or the quad's depth outside the clip volume: GL clips it
    f.ok = w > 0.f && fabsf(pz / w) <= 1.f;
    return f;
}

// Fragment shader at relCoord (u, v): false when discarded; the 24-bit depth
// and the attenuation otherwise.
__device__ __forceinline__ bool fragment(const Camera& c, const Frag& f, float R, float u, float v, unsigned int& d24,
                                         float& atten) {
    const float norm = u * u + v * v;
    if (norm > 1.f) return false;
    const float nz = sqrtf(1.f - norm);
    const float zEye = f.ez + R * nz;
    const float z = -c.p[10] - c.p[11] / zEye;
    const float zc = fminf(fmaxf(z, 0.f), 1.f);
    d24 = __float2uint_rn(zc * 16777215.f);
    atten = 0.9f + 0.1f * fmaxf(0.f, nz);
    return true;
}

// Pixel centre (i + 0.5, j + 0.5) of window coordinates -> NDC.
__device__ __forceinline__ float ndc(int i, int size) { return ((float)i + 0.5f) * 2.f / (float)size - 1.f; }

__device__ __forceinline__ void locate(const Passes& P, int idx, int& pass, int& k) {
    pass = 0;
    while (pass + 1 < P.num && idx >= P.p[pass + 1].base) pass++;
    k = idx - P.p[pass].base;
}

__global__ void k_splat(Passes P, int total, Camera cam, int W, int H, unsigned long long* __restrict__ keys) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= total) return;
    int pass, k;
    locate(P, idx, pass, k);
    const Pass& q = P.p[pass];
    const float4 x = q.pos[q.ids ? q.ids[k] : k];
    const Frag f = project(cam, x, q.radius);
    if (!f.ok || !(f.dx > 0.f) || !(f.dy > 0.f)) return;
    // window-space extent; the pixels whose centres fall inside the quad
    const float xl = (f.cx - f.dx + 1.f) * 0.5f * (float)W, xr = (f.cx + f.dx + 1.f) * 0.5f * (float)W;
    const float yl = (f.cy - f.dy + 1.f) * 0.5f * (float)H, yr = (f.cy + f.dy + 1.f) * 0.5f * (float)H;
    const int i0 = max((int)ceilf(xl - 0.5f), 0), i1 = min((int)ceilf(xr - 0.5f) - 1, W - 1);
    const int j0 = max((int)ceilf(yl - 0.5f), 0), j1 = min((int)ceilf(yr - 0.5f) - 1, H - 1);
    for (int j = j0; j <= j1; j++) {
        const float v = (ndc(j, H) - f.cy) / f.dy;
        for (int i = i0; i <= i1; i++) {
            const float u = (ndc(i, W) - f.cx) / f.dx;
            unsigned int d24;
            float atten;
            if (!fragment(cam, f, q.radius, u, v, d24, atten)) continue;
            const unsigned long long key = ((unsigned long long)d24 << 32) | (unsigned int)idx;
            // window row j is image row H - 1 - j
            atomicMin(keys + (size_t)(H - 1 - j) * W + i, key);
        }
    }
}

__global__ void k_shade(Passes P, Camera cam, int W, int H, const unsigned long long* __restrict__ keys,
                        uchar4* __restrict__ rgba, float* __restrict__ depth) {
    const int pix = blockIdx.x * blockDim.x + threadIdx.x;
    if (pix >= W * H) return;
    const unsigned long long key = keys[pix];
    uchar4 out = make_uchar4(255, 255, 255, 255);  // glClearColor(1, 1, 1, 1)
    float dz = 1.f;
    if (key != EMPTY_KEY) {
        const int idx = (int)(unsigned int)(key & 0xffffffffull);
        int pass, k;
        locate(P, idx, pass, k);
        const Pass& q = P.p[pass];
        const float4 x = q.pos[q.ids ? q.ids[k] : k];
        const Frag f = project(cam, x, q.radius);
        const int i = pix % W, j = H - 1 - pix / W;
        const float u = (ndc(i, W) - f.cx) / f.dx, v = (ndc(j, H) - f.cy) / f.dy;
        unsigned int d24;
        float atten = 1.f;
        fragment(cam, f, q.radius, u, v, d24, atten);
        // unsigned normalised 8-bit conversion of the fragment colour
        auto un8 = [](float c) { return (unsigned char)__float2uint_rn(fminf(fmaxf(c, 0.f), 1.f) * 255.f); };
        out = make_uchar4(un8(atten * q.rgb[0]), un8(atten * q.rgb[1]), un8(atten * q.rgb[2]), un8(atten));
        dz = (float)(key >> 32) / 16777215.f;
    }
    rgba[pix] = out;
    if (depth) depth[pix] = dz;
}

}  // namespace
}  // namespace sph

using namespace sph;

extern "C" {

sph_status sph_camera_look_at(sph_camera* cam, const float eye[3], const float centre[3], const float up[3]) {
    if (!cam || !eye || !centre || !up) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "NULL argument");
    // camera base u, v, n (cgtkGLLookAt, cgtk/src/opengl.c:10-46)
    float n[3] = {centre[0] - eye[0], centre[1] - eye[1], centre[2] - eye[2]};
    auto normalise = [](float* a) {
        const float l = sqrtf(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
        if (l > 0.f)
            for (int k = 0; k < 3; k++) a[k] /= l;
    };
    auto cross = [](const float* a, const float* b, float* c) {
        c[0] = a[1] * b[2] - a[2] * b[1];
        c[1] = a[2] * b[0] - a[0] * b[2];
        c[2] = a[0] * b[1] - a[1] * b[0];
    };
    normalise(n);
    float u[3], v[3];
    cross(n, up, u);
    normalise(u);
    cross(u, n, v);
    float* m = cam->view;
    for (int a = 0; a < 3; a++) {
        m[4 * a + 0] = u[a];
        m[4 * a + 1] = v[a];
        m[4 * a + 2] = -n[a];
        m[4 * a + 3] = 0.f;
    }
    m[12] = -(u[0] * eye[0] + u[1] * eye[1] + u[2] * eye[2]);
    m[13] = -(v[0] * eye[0] + v[1] * eye[1] + v[2] * eye[2]);
    m[14] = n[0] * eye[0] + n[1] * eye[1] + n[2] * eye[2];
    m[15] = 1.f;
    return SPH_OK;
}

sph_status sph_camera_perspective(sph_camera* cam, float fovy, float aspect, float znear, float zfar) {
    if (!cam) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "NULL argument");
    if (!(znear > 0.f) || !(zfar > znear) || !(aspect > 0.f) || !(fovy > 0.f && fovy < 180.f))
        SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "invalid perspective");
    // cgtkGLPerspective + cgtkGLFrustum (cgtk/src/opengl.c:48-78)
    const float t = tanf((fovy / 2.0f) * (3.141593f / 180.f));
    const float h = znear * t, w = h * aspect;
    const float l = -w, r = w, b = -h, tp = h;
    float* m = cam->proj;
    for (int k = 0; k < 16; k++) m[k] = 0.f;
    m[0] = 2.f * znear / (r - l);
    m[5] = 2.f * znear / (tp - b);
    m[8] = (r + l) / (r - l);
    m[9] = (tp + b) / (tp - b);
    m[10] = (zfar + znear) / (znear - zfar);
    m[11] = -1.f;
    m[14] = -2.f * zfar * znear / (zfar - znear);
    return SPH_OK;
}

sph_status sph_render(sph_handle s, const sph_camera* cam, int width, int height, int what, unsigned char* rgba,
                      float* depth) {
    if (!s || !cam || !rgba) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "NULL argument");
    if (width <= 0 || height <= 0 || (long long)width * height > (1ll << 26))
        SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "image size must be positive and at most 2^26 pixels");
    if (what != SPH_RENDER_PARTICLES && what != SPH_RENDER_TWO_SCALE && what != SPH_RENDER_SUB_PARTICLES)
        SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "unknown render mode");
    sph_status st = latched_status(s);
    if (st) return st;
    cudaStream_t q = s->stream;
    // ParticleSimulation::GetParticleRadius (particle_simulation.cu:2227-2236)
    const float R = powf((float)((3.0 * s->P.fluidVolume) / (4.0 * M_PI * s->P.numParticles)), 1.0f / 3.0f);
    Passes P{};
    float4* absPos = nullptr;
    const float4* coarse = s->pos;
    if (s->O.cellRelative) {
        SPH_CUDA(dalloc(&absPos, (size_t)s->n));
        launch_rel_to_abs(s->n, s->pos, grid_of(s), nullptr, 0, absPos, q);
        coarse = absPos;
    }
    int counts[4] = {0, 0, s->n, 0};  // split, boundary, default, children
    if (what != SPH_RENDER_PARTICLES) {
        if (!s->tsReady) {
            if (absPos) cudaFree(absPos);
            SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "no two-scale step has run yet");
        }
        SPH_CUDA(cudaMemcpyAsync(counts, s->ts.counts, sizeof(int) * 4, cudaMemcpyDeviceToHost, q));
        SPH_CUDA(cudaStreamSynchronize(q));
    }
    auto add = [&](const float4* pos, const int* ids, int count, float radius, float r, float g, float b) {
        Pass& p = P.p[P.num];
        p.pos = pos;
        p.ids = ids;
        p.count = count;
        p.base = P.num ? P.p[P.num - 1].base + P.p[P.num - 1].count : 0;
        p.radius = radius;
        p.rgb[0] = r;
        p.rgb[1] = g;
        p.rgb[2] = b;
        P.num++;
    };
    // the draw calls of TwoScaleStateSub::renderLow / render / renderRegularSubParticles
    if (what == SPH_RENDER_PARTICLES) {
        add(coarse, nullptr, s->n, R, 0.f, 0.f, 0.9f);
    } else {
        const int regular = 8 * counts[0], boundary = 8 * counts[1];
        if (what == SPH_RENDER_TWO_SCALE) add(coarse, s->ts.defaultIds, counts[2], R, 0.f, 0.f, 0.9f);
        add(s->ts.subPos, s->ts.subIds, regular, 0.5f * R, 0.9f, 0.9f, 0.f);
        add(s->ts.subPos, s->ts.subIds + regular, boundary, 0.5f * R, 0.9f, 0.f, 0.f);
    }
    const int total = P.p[P.num - 1].base + P.p[P.num - 1].count;
    Camera c;
    for (int k = 0; k < 16; k++) {
        c.v[k] = cam->view[k];
        c.p[k] = cam->proj[k];
    }
    const size_t pixels = (size_t)width * height;
    unsigned long long* keys = nullptr;
    uchar4* img = nullptr;
    float* dep = nullptr;
    cudaError_t e = cudaMalloc(&keys, sizeof(unsigned long long) * pixels);
    if (e == cudaSuccess) e = cudaMalloc(&img, sizeof(uchar4) * pixels);
    if (e == cudaSuccess && depth) e = cudaMalloc(&dep, sizeof(float) * pixels);
    if (e == cudaSuccess) e = cudaMemsetAsync(keys, 0xff, sizeof(unsigned long long) * pixels, q);
    if (e == cudaSuccess && total > 0) {
        k_splat<<<(total + 127) / 128, 128, 0, q>>>(P, total, c, width, height, keys);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        k_shade<<<(unsigned int)((pixels + 255) / 256), 256, 0, q>>>(P, c, width, height, keys, img, dep);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(rgba, img, sizeof(uchar4) * pixels, cudaMemcpyDeviceToHost, q);
    if (e == cudaSuccess && depth) e = cudaMemcpyAsync(depth, dep, sizeof(float) * pixels, cudaMemcpyDeviceToHost, q);
    if (e == cudaSuccess) e = cudaStreamSynchronize(q);
    cudaFree(keys);
    cudaFree(img);
    if (dep) cudaFree(dep);
    if (absPos) cudaFree(absPos);
    SPH_CUDA(e);
    return latched_status(s);
}

sph_status sph_image_save_ppm(const char* path, const unsigned char* rgba, int width, int height) {
    if (!path || !rgba || width <= 0 || height <= 0) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "invalid argument");
    // PortablePixmap::save's layout (portable_pixmap.cpp:23-40): ASCII P3,
    // maximum 255, one value per line, rows top to bottom
    FILE* f = fopen(path, "w");
    if (!f) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "cannot open the file for writing");
    fprintf(f, "P3\n%d %d\n255\n", width, height);
    const size_t pixels = (size_t)width * height;
    for (size_t k = 0; k < pixels; k++)
        fprintf(f, "%u\n%u\n%u\n", rgba[4 * k], rgba[4 * k + 1], rgba[4 * k + 2]);
    const bool ok = fclose(f) == 0;
    if (!ok) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "write failed");
    return SPH_OK;
}

}  // extern "C"
