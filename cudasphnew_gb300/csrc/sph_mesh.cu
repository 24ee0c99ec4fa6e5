// Mesh signed distance fields on the GPU, the boundary-map text format and an
// OBJ reader (BoundaryMap::AddCanvas / computeSignedDistanceField,
// boundary_map.cpp:50-95, 351-470; PointInMeshTest, point_in_mesh_test.cpp:
// 31-206; BoundaryMap::Save / Load, boundary_map.cpp:161-287).
//
// Distance.  Every grid node takes the smallest distance to the mesh's
// triangles; the reference visits, per triangle, the nodes of the triangle's
// bounding box grown by maxDist + dx and keeps a node whose distance is at
// most maxDist = max(restDistance, compactSupport), replacing an earlier
// value only when strictly smaller (so the first triangle wins a tie).  Here
// each node visits the triangles in order with the same strict rule; a
// triangle whose bounding box grown by maxDist misses the node cannot be
// within maxDist of it, so the band is the same.  The closest point on a
// triangle is found by Voronoi-region classification (Ericson, Real-Time
// Collision Detection, section 5.1.5) in double precision; the reference
// calls Wm5::DistPoint3Triangle3f (WildMagic 5), which minimises the same
// distance.  The node's normal is (x - closest point) / |x - closest point|,
// as at boundary_map.cpp:536-550.
//
// Sign.  Inside nodes are negated (boundary_map.cpp:455-469).  The reference
// decides inside by the parity of a near-vertical ray's triangle crossings,
// with a tilt drawn from std::rand seeded by the clock (point_in_mesh_test.cpp:
// 67-78), so its result is not reproducible; here the tilt is fixed
// (0.3137 dx, 0.2718 dx per mesh height) and the crossing test is
// Moller-Trumbore's (1997) in double precision.  Nodes outside the mesh's
// bounding box are outside (:33-36).  Every node gets a sign, not only the
// band's: nodes beyond the band hold +-maxDist.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "sph_sim.h"

namespace sph {

namespace {

__host__ __device__ inline void sub3(const double* a, const double* b, double* r) {
    r[0] = a[0] - b[0];
    r[1] = a[1] - b[1];
    r[2] = a[2] - b[2];
}
__host__ __device__ inline double dot3(const double* a, const double* b) {
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

// Closest point q on triangle (a, b, c) to p (Ericson 5.1.5).
__host__ __device__ void closest_on_triangle(const double* p, const double* a, const double* b, const double* c,
                                             double* q) {
    double ab[3], ac[3], ap[3];
    sub3(b, a, ab);
    sub3(c, a, ac);
    sub3(p, a, ap);
    const double d1 = dot3(ab, ap), d2 = dot3(ac, ap);
    if (d1 <= 0.0 && d2 <= 0.0) {
        q[0] = a[0], q[1] = a[1], q[2] = a[2];
        return;
    }
    double bp[3];
    sub3(p, b, bp);
    const double d3 = dot3(ab, bp), d4 = dot3(ac, bp);
    if (d3 >= 0.0 && d4 <= d3) {
        q[0] = b[0], q[1] = b[1], q[2] = b[2];
        return;
    }
    const double vc = d1 * d4 - d3 * d2;
    if (vc <= 0.0 && d1 >= 0.0 && d3 <= 0.0) {
        const double v = d1 / (d1 - d3);
        for (int k = 0; k < 3; k++) q[k] = a[k] + v * ab[k];
        return;
    }
    double cp[3];
    sub3(p, c, cp);
    const double d5 = dot3(ab, cp), d6 = dot3(ac, cp);
    if (d6 >= 0.0 && d5 <= d6) {
        q[0] = c[0], q[1] = c[1], q[2] = c[2];
        return;
    }
    const double vb = d5 * d2 - d1 * d6;
    if (vb <= 0.0 && d2 >= 0.0 && d6 <= 0.0) {
        const double w = d2 / (d2 - d6);
        for (int k = 0; k < 3; k++) q[k] = a[k] + w * ac[k];
        return;
    }
    const double va = d3 * d6 - d5 * d4;
    if (va <= 0.0 && (d4 - d3) >= 0.0 && (d5 - d6) >= 0.0) {
        const double w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
        for (int k = 0; k < 3; k++) q[k] = b[k] + w * (c[k] - b[k]);
        return;
    }
    const double den = 1.0 / (va + vb + vc);
    const double v = vb * den, w = vc * den;
    for (int k = 0; k < 3; k++) q[k] = a[k] + ab[k] * v + ac[k] * w;
}

// Does the ray o + t d (t > 0) cross triangle (a, b, c)?  Moller-Trumbore.
__host__ __device__ bool ray_crosses(const double* o, const double* d, const double* a, const double* b,
                                     const double* c) {
    double e1[3], e2[3], s[3];
    sub3(b, a, e1);
    sub3(c, a, e2);
    const double pv[3] = {d[1] * e2[2] - d[2] * e2[1], d[2] * e2[0] - d[0] * e2[2], d[0] * e2[1] - d[1] * e2[0]};
    const double det = dot3(e1, pv);
    if (det == 0.0) return false;  // ray parallel to the triangle's plane
    const double inv = 1.0 / det;
    sub3(o, a, s);
    const double u = dot3(s, pv) * inv;
    if (u < 0.0 || u > 1.0) return false;
    const double qv[3] = {s[1] * e1[2] - s[2] * e1[1], s[2] * e1[0] - s[0] * e1[2], s[0] * e1[1] - s[1] * e1[0]};
    const double v = dot3(d, qv) * inv;
    if (v < 0.0 || u + v > 1.0) return false;
    return dot3(e2, qv) * inv > 0.0;
}

struct SdfArgs {
    const float* verts;
    const unsigned int* faces;
    unsigned int numFaces;
    float origin[3];
    float dx;
    unsigned int dims[3];
    float maxDist;
    float bbLo[3], bbHi[3];  // the mesh's bounding box
    double ray[3];           // the parity ray's direction
};

__device__ void load_tri(const SdfArgs& A, unsigned int m, double* a, double* b, double* c) {
    const unsigned int i0 = A.faces[3 * m], i1 = A.faces[3 * m + 1], i2 = A.faces[3 * m + 2];
    for (int k = 0; k < 3; k++) {
        a[k] = A.verts[3 * i0 + k];
        b[k] = A.verts[3 * i1 + k];
        c[k] = A.verts[3 * i2 + k];
    }
}

__global__ void k_mesh_sdf(SdfArgs A, float* __restrict__ dist, float* __restrict__ normal) {
    const size_t n = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t total = (size_t)A.dims[0] * A.dims[1] * A.dims[2];
    if (n >= total) return;
    const unsigned int i = (unsigned int)(n % A.dims[0]);
    const unsigned int j = (unsigned int)((n / A.dims[0]) % A.dims[1]);
    const unsigned int k = (unsigned int)(n / ((size_t)A.dims[0] * A.dims[1]));
    // node position formed in float, as x0 + i*mDx (boundary_map.cpp:400-402)
    const float xf[3] = {__fadd_rn(A.origin[0], __fmul_rn((float)i, A.dx)),
                         __fadd_rn(A.origin[1], __fmul_rn((float)j, A.dx)),
                         __fadd_rn(A.origin[2], __fmul_rn((float)k, A.dx))};
    const double x[3] = {xf[0], xf[1], xf[2]};
    const double md = A.maxDist;
    double best = 1e300, q[3] = {0.0, 0.0, 0.0};
    for (unsigned int m = 0; m < A.numFaces; m++) {
        double a[3], b[3], c[3];
        load_tri(A, m, a, b, c);
        bool far = false;
        for (int e = 0; e < 3 && !far; e++) {
            const double lo = fmin(a[e], fmin(b[e], c[e])) - md, hi = fmax(a[e], fmax(b[e], c[e])) + md;
            far = x[e] < lo || x[e] > hi;
        }
        if (far) continue;
        double p[3];
        closest_on_triangle(x, a, b, c, p);
        double r[3];
        sub3(x, p, r);
        const double d = sqrt(dot3(r, r));
        if (d < best) {  // strictly smaller: the first triangle keeps a tie
            best = d;
            q[0] = p[0], q[1] = p[1], q[2] = p[2];
        }
    }
    const bool band = best <= md;
    // parity of the ray's crossings: only triangles whose xy box meets the
    // ray's xy footprint inside the mesh's z range can be crossed
    bool inside = false;
    const bool inBox = x[0] >= A.bbLo[0] && x[0] <= A.bbHi[0] && x[1] >= A.bbLo[1] && x[1] <= A.bbHi[1] &&
                       x[2] >= A.bbLo[2] && x[2] <= A.bbHi[2];
    if (inBox) {
        const double tmax = (A.bbHi[2] - x[2]) / A.ray[2];
        const double fx0 = fmin(x[0], x[0] + A.ray[0] * tmax), fx1 = fmax(x[0], x[0] + A.ray[0] * tmax);
        const double fy0 = fmin(x[1], x[1] + A.ray[1] * tmax), fy1 = fmax(x[1], x[1] + A.ray[1] * tmax);
        unsigned int cnt = 0;
        for (unsigned int m = 0; m < A.numFaces; m++) {
            double a[3], b[3], c[3];
            load_tri(A, m, a, b, c);
            if (fmax(a[0], fmax(b[0], c[0])) < fx0 || fmin(a[0], fmin(b[0], c[0])) > fx1) continue;
            if (fmax(a[1], fmax(b[1], c[1])) < fy0 || fmin(a[1], fmin(b[1], c[1])) > fy1) continue;
            if (fmax(a[2], fmax(b[2], c[2])) < x[2]) continue;
            cnt += ray_crosses(x, A.ray, a, b, c) ? 1u : 0u;
        }
        inside = (cnt & 1u) != 0u;
    }
    const double mag = band ? best : md;
    dist[n] = (float)(inside ? -mag : mag);
    if (normal) {
        float nv[3] = {0.f, 0.f, 0.f};
        if (band && best > 0.0) {
            for (int e = 0; e < 3; e++) nv[e] = (float)((x[e] - q[e]) / best);
        }
        normal[3 * n] = nv[0];
        normal[3 * n + 1] = nv[1];
        normal[3 * n + 2] = nv[2];
    }
}

}  // namespace

}  // namespace sph

using namespace sph;

namespace {

// One OBJ face index: "i", "i/t", "i//n", "i/t/n"; 1-based or negative.
bool obj_index(const char* tok, long nv, long* out) {
    char* end = nullptr;
    const long v = std::strtol(tok, &end, 10);
    if (end == tok || v == 0) return false;
    *out = v > 0 ? v - 1 : nv + v;
    return *out >= 0 && *out < nv;
}

sph_status sdf_compute(const sph_mesh* mesh, const float origin[3], float dx, const unsigned int dims[3],
                       float restDistance, float compactSupport, sph_sdf_grid* out) {
    if (!mesh || !out || !mesh->vertices || !mesh->faces) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "NULL argument");
    if (mesh->numFaces == 0 || mesh->numVertices == 0) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "empty mesh");
    if (!(dx > 0.0f)) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "dx must be positive");
    for (unsigned int f = 0; f < 3 * mesh->numFaces; f++)
        if (mesh->faces[f] >= mesh->numVertices) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "face index out of range");
    const double total = (double)dims[0] * dims[1] * dims[2];
    if (dims[0] == 0 || dims[1] == 0 || dims[2] == 0 || total > 512.0 * 1024 * 1024)
        SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "grid must have 1 .. 2^29 nodes");
    std::memset(out, 0, sizeof(*out));
    const size_t n = (size_t)total;
    SdfArgs A{};
    A.numFaces = mesh->numFaces;
    A.dx = dx;
    A.maxDist = restDistance > compactSupport ? restDistance : compactSupport;
    for (int a = 0; a < 3; a++) {
        A.origin[a] = origin[a];
        A.dims[a] = dims[a];
        A.bbLo[a] = A.bbHi[a] = mesh->vertices[a];
    }
    for (unsigned int v = 0; v < mesh->numVertices; v++)
        for (int a = 0; a < 3; a++) {
            A.bbLo[a] = std::fmin(A.bbLo[a], mesh->vertices[3 * v + a]);
            A.bbHi[a] = std::fmax(A.bbHi[a], mesh->vertices[3 * v + a]);
        }
    const double height = std::fmax((double)A.bbHi[2] - A.bbLo[2], (double)dx);
    A.ray[0] = 0.3137 * dx;
    A.ray[1] = 0.2718 * dx;
    A.ray[2] = height;
    float *dv = nullptr, *dd = nullptr, *dn = nullptr;
    unsigned int* df = nullptr;
    cudaStream_t q = nullptr;
    auto done = [&]() {
        void* p[] = {dv, dd, dn, df};
        for (void* x : p)
            if (x) cudaFree(x);
        if (q) cudaStreamDestroy(q);
    };
    cudaError_t e = cudaStreamCreateWithFlags(&q, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = dalloc(&dv, (size_t)mesh->numVertices * 3);
    if (e == cudaSuccess) e = dalloc(&df, (size_t)mesh->numFaces * 3);
    if (e == cudaSuccess) e = dalloc(&dd, n);
    if (e == cudaSuccess) e = dalloc(&dn, 3 * n);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(dv, mesh->vertices, sizeof(float) * 3 * mesh->numVertices, cudaMemcpyHostToDevice, q);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(df, mesh->faces, sizeof(unsigned int) * 3 * mesh->numFaces, cudaMemcpyHostToDevice, q);
    if (e == cudaSuccess) {
        A.verts = dv;
        A.faces = df;
        k_mesh_sdf<<<(unsigned int)((n + 127) / 128), 128, 0, q>>>(A, dd, dn);
        e = cudaGetLastError();
    }
    float* hd = nullptr;
    float* hn = nullptr;
    if (e == cudaSuccess) {
        hd = static_cast<float*>(std::malloc(sizeof(float) * n));
        hn = static_cast<float*>(std::malloc(sizeof(float) * 3 * n));
        if (!hd || !hn) e = cudaErrorMemoryAllocation;
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(hd, dd, sizeof(float) * n, cudaMemcpyDeviceToHost, q);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hn, dn, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost, q);
    if (e == cudaSuccess) e = cudaStreamSynchronize(q);
    done();
    if (e != cudaSuccess) {
        std::free(hd);
        std::free(hn);
        SPH_CUDA(e);
    }
    for (int a = 0; a < 3; a++) {
        out->origin[a] = origin[a];
        out->dims[a] = dims[a];
    }
    out->dx = dx;
    out->restDistance = restDistance;
    out->compactSupport = compactSupport;
    out->maxDist = A.maxDist;
    out->distance = hd;
    out->normal = hn;
    return SPH_OK;
}

}  // namespace

extern "C" {

sph_status sph_obj_load(const char* path, sph_mesh* out) {
    if (!path || !out) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "NULL argument");
    std::memset(out, 0, sizeof(*out));
    FILE* f = std::fopen(path, "r");
    if (!f) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, std::string("cannot open ") + path);
    std::vector<float> v;
    std::vector<unsigned int> tri;
    char line[4096];
    bool bad = false;
    while (std::fgets(line, sizeof(line), f)) {
        if (line[0] == 'v' && (line[1] == ' ' || line[1] == '\t')) {
            float x, y, z;
            if (std::sscanf(line + 2, "%f %f %f", &x, &y, &z) != 3) {
                bad = true;
                break;
            }
            v.push_back(x);
            v.push_back(y);
            v.push_back(z);
        } else if (line[0] == 'f' && (line[1] == ' ' || line[1] == '\t')) {
            std::vector<long> idx;
            char* save = nullptr;
            for (char* tok = strtok_r(line + 2, " \t\r\n", &save); tok; tok = strtok_r(nullptr, " \t\r\n", &save)) {
                long k;
                if (!obj_index(tok, (long)(v.size() / 3), &k)) {
                    bad = true;
                    break;
                }
                idx.push_back(k);
            }
            if (bad || idx.size() < 3) {
                bad = true;
                break;
            }
            for (size_t t = 1; t + 1 < idx.size(); t++) {  // fan
                tri.push_back((unsigned int)idx[0]);
                tri.push_back((unsigned int)idx[t]);
                tri.push_back((unsigned int)idx[t + 1]);
            }
        }
    }
    std::fclose(f);
    if (bad) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, std::string("malformed OBJ record in ") + path);
    if (v.empty() || tri.empty()) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, std::string("no triangles in ") + path);
    out->vertices = static_cast<float*>(std::malloc(sizeof(float) * v.size()));
    out->faces = static_cast<unsigned int*>(std::malloc(sizeof(unsigned int) * tri.size()));
    if (!out->vertices || !out->faces) {
        sph_mesh_free(out);
        SPH_FAIL(SPH_ERR_OUT_OF_MEMORY, "host allocation failed");
    }
    std::memcpy(out->vertices, v.data(), sizeof(float) * v.size());
    std::memcpy(out->faces, tri.data(), sizeof(unsigned int) * tri.size());
    out->numVertices = (unsigned int)(v.size() / 3);
    out->numFaces = (unsigned int)(tri.size() / 3);
    return SPH_OK;
}

void sph_mesh_free(sph_mesh* m) {
    if (!m) return;
    std::free(m->vertices);
    std::free(m->faces);
    std::memset(m, 0, sizeof(*m));
}

sph_status sph_sdf_from_mesh(const sph_mesh* mesh, float restDistance, float compactSupport, float dx,
                             sph_sdf_grid* out) {
    if (!mesh || !mesh->vertices || mesh->numVertices == 0) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "empty mesh");
    if (!(dx > 0.0f)) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "dx must be positive");
    // AddCanvas (boundary_map.cpp:56-80): the mesh's bounding box, ceil(extent/dx)
    // intervals per axis
    float lo[3], hi[3];
    for (int a = 0; a < 3; a++) lo[a] = hi[a] = mesh->vertices[a];
    for (unsigned int i = 0; i < mesh->numVertices; i++)
        for (int a = 0; a < 3; a++) {
            lo[a] = std::fmin(lo[a], mesh->vertices[3 * i + a]);
            hi[a] = std::fmax(hi[a], mesh->vertices[3 * i + a]);
        }
    unsigned int dims[3];
    for (int a = 0; a < 3; a++) dims[a] = (unsigned int)std::ceil((hi[a] - lo[a]) / dx) + 1u;
    return sdf_compute(mesh, lo, dx, dims, restDistance, compactSupport, out);
}

sph_status sph_sdf_from_mesh_on_grid(const sph_mesh* mesh, const float origin[3], float dx,
                                     const unsigned int dims[3], float restDistance, float compactSupport,
                                     sph_sdf_grid* out) {
    if (!origin || !dims) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "NULL argument");
    return sdf_compute(mesh, origin, dx, dims, restDistance, compactSupport, out);
}

void sph_sdf_free(sph_sdf_grid* g) {
    if (!g) return;
    std::free(g->distance);
    std::free(g->normal);
    g->distance = nullptr;
    g->normal = nullptr;
}

sph_status sph_sdf_save(const sph_sdf_grid* g, const char* path) {
    if (!g || !path || !g->distance) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "NULL argument");
    FILE* f = std::fopen(path, "w");
    if (!f) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, std::string("cannot write ") + path);
    const size_t n = (size_t)g->dims[0] * g->dims[1] * g->dims[2];
    size_t band = 0;
    for (size_t k = 0; k < n; k++) band += std::fabs(g->distance[k]) < g->maxDist || (g->normal && (g->normal[3 * k] != 0.f || g->normal[3 * k + 1] != 0.f || g->normal[3 * k + 2] != 0.f));
    // header (boundary_map.cpp:173-187): restDistance, compactSupport, maxDist,
    // dx, domain corners, node counts, total samples, stored coordinates
    std::fprintf(f, "%.9g\n%.9g\n%.9g\n%.9g\n", g->restDistance, g->compactSupport, g->maxDist, g->dx);
    for (int a = 0; a < 3; a++) std::fprintf(f, "%.9g\n", g->origin[a]);
    for (int a = 0; a < 3; a++) std::fprintf(f, "%.9g\n", g->origin[a] + (float)(g->dims[a] - 1) * g->dx);
    std::fprintf(f, "%u\n%u\n%u\n%zu\n%zu\n", g->dims[0], g->dims[1], g->dims[2], n, band);
    // band nodes (|distance| < maxDist, or a surface normal) in node order:
    // i, j, k, distance, normal (:188-208; the reference lists them in the
    // order its sparse map received them, which Load does not depend on)
    for (size_t k = 0; k < n; k++) {
        const bool nz = g->normal && (g->normal[3 * k] != 0.f || g->normal[3 * k + 1] != 0.f || g->normal[3 * k + 2] != 0.f);
        if (!(std::fabs(g->distance[k]) < g->maxDist || nz)) continue;
        const unsigned int i = (unsigned int)(k % g->dims[0]);
        const unsigned int j = (unsigned int)((k / g->dims[0]) % g->dims[1]);
        const unsigned int kk = (unsigned int)(k / ((size_t)g->dims[0] * g->dims[1]));
        const float* nv = g->normal ? g->normal + 3 * k : nullptr;
        std::fprintf(f, "%u\n%u\n%u\n%.9g\n%.9g\n%.9g\n%.9g\n", i, j, kk, g->distance[k], nv ? nv[0] : 0.f,
                     nv ? nv[1] : 0.f, nv ? nv[2] : 0.f);
    }
    const bool ok = std::fflush(f) == 0;
    std::fclose(f);
    if (!ok) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, std::string("write failed: ") + path);
    return SPH_OK;
}

sph_status sph_sdf_load(const char* path, sph_sdf_grid* out) {
    if (!path || !out) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "NULL argument");
    std::memset(out, 0, sizeof(*out));
    FILE* f = std::fopen(path, "r");
    if (!f) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, std::string("cannot open ") + path);
    float v1[3], v2[3];
    unsigned int dims[3];
    unsigned long long total = 0, count = 0;
    bool ok = std::fscanf(f, "%f %f %f %f", &out->restDistance, &out->compactSupport, &out->maxDist, &out->dx) == 4 &&
              std::fscanf(f, "%f %f %f %f %f %f", &v1[0], &v1[1], &v1[2], &v2[0], &v2[1], &v2[2]) == 6 &&
              std::fscanf(f, "%u %u %u %llu %llu", &dims[0], &dims[1], &dims[2], &total, &count) == 5;
    ok = ok && dims[0] && dims[1] && dims[2] && total == (unsigned long long)dims[0] * dims[1] * dims[2] &&
         total <= 512ull * 1024 * 1024 && count <= total;
    if (!ok) {
        std::fclose(f);
        SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, std::string("malformed boundary map header in ") + path);
    }
    const size_t n = (size_t)total;
    out->distance = static_cast<float*>(std::malloc(sizeof(float) * n));
    out->normal = static_cast<float*>(std::calloc(3 * n, sizeof(float)));
    if (!out->distance || !out->normal) {
        std::fclose(f);
        sph_sdf_free(out);
        SPH_FAIL(SPH_ERR_OUT_OF_MEMORY, "host allocation failed");
    }
    // nodes not listed hold the rest distance with a zero normal (:248-252)
    for (size_t k = 0; k < n; k++) out->distance[k] = out->restDistance;
    for (unsigned long long c = 0; c < count && ok; c++) {
        unsigned int ijk[3];
        float d, nx, ny, nz;
        ok = std::fscanf(f, "%u %u %u %f %f %f %f", &ijk[0], &ijk[1], &ijk[2], &d, &nx, &ny, &nz) == 7 &&
             ijk[0] < dims[0] && ijk[1] < dims[1] && ijk[2] < dims[2];
        if (!ok) break;
        const size_t k = ijk[0] + (size_t)dims[0] * (ijk[1] + (size_t)dims[1] * ijk[2]);
        out->distance[k] = d;
        out->normal[3 * k] = nx;
        out->normal[3 * k + 1] = ny;
        out->normal[3 * k + 2] = nz;
    }
    std::fclose(f);
    if (!ok) {
        sph_sdf_free(out);
        SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, std::string("malformed boundary map record in ") + path);
    }
    for (int a = 0; a < 3; a++) {
        out->origin[a] = v1[a];
        out->dims[a] = dims[a];
    }
    return SPH_OK;
}

}  // extern "C"
