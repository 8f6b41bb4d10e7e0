// nw_defects.cu — +1/2 / -1/2 defects of the director field on the device
// (include/nwgb.h, "topological defects"): the grid search of
// analysis/find_defects.py (nw_find_defects) and the sampling search of
// analysis/defects.py (nw_sample_defects, one block per sample point, at the
// end of this file).
//
// The grid search runs three kernels: the beads' bounding box (float min/max through order-
// preserving integer atomics); every bead adds cos 2a and sin 2a of its
// tangent angle a to its grid cell as 2^30 fixed-point integers (integer
// atomics: the sums, and so every later result, are the same whatever the
// thread order); every interior cell sums the director's rotation along the
// ring of its eight neighbours and lists itself when the total exceeds
// pi - pi/16 in magnitude.  The host merges touching marked cells of one sign
// as the reference's analysis does (analysis/find_defects.py:126-160).
//
// The cell of a bead is floor((r - min) / cell_size) in double precision,
// the reference's float64 arithmetic on the same float32 positions, so beads
// on a cell edge land where they land there.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "nw_engine.h"
#include "nw_system.h"

namespace {

constexpr double kFix = 1073741824.0;  // 2^30
constexpr float kPi = 3.14159265358979323846f;

struct DefectGrid {
    uint32_t nx, ny;
    double cs, ox, oy;
};

// float <-> uint32 keeping the order, for min/max by integer atomics
__device__ __forceinline__ uint32_t ord_key(float f)
{
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
inline float ord_val(uint32_t k)
{
    const uint32_t u = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

__global__ void __launch_bounds__(256) defect_bounds_kernel(const float4* __restrict__ pos, uint32_t nb,
                                                            uint32_t* __restrict__ box)
{
    __shared__ uint32_t s_k[4][8];
    uint32_t k[4] = {0xffffffffu, 0xffffffffu, 0u, 0u};  // lo x, lo y, hi x, hi y
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nb; i += gridDim.x * blockDim.x) {
        const float4 r = pos[i];
        const uint32_t kx = ord_key(r.x), ky = ord_key(r.y);
        k[0] = min(k[0], kx), k[1] = min(k[1], ky), k[2] = max(k[2], kx), k[3] = max(k[3], ky);
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        k[0] = min(k[0], __shfl_xor_sync(0xffffffffu, k[0], o));
        k[1] = min(k[1], __shfl_xor_sync(0xffffffffu, k[1], o));
        k[2] = max(k[2], __shfl_xor_sync(0xffffffffu, k[2], o));
        k[3] = max(k[3], __shfl_xor_sync(0xffffffffu, k[3], o));
    }
    const uint32_t w = threadIdx.x >> 5;
    if ((threadIdx.x & 31u) == 0)
        for (int a = 0; a < 4; ++a) s_k[a][w] = k[a];
    __syncthreads();
    if (threadIdx.x < 4) {  // one atomic per value and block
        const uint32_t a = threadIdx.x;
        uint32_t v = s_k[a][0];
        for (uint32_t q = 1; q < (blockDim.x >> 5); ++q) v = a < 2 ? min(v, s_k[a][q]) : max(v, s_k[a][q]);
        if (a < 2) atomicMin(box + a, v);
        else atomicMax(box + a, v);
    }
}

__global__ void __launch_bounds__(256) defect_bin_kernel(const nw::DevParams P, const float4* __restrict__ pos,
                                                         DefectGrid G, bool min_image, long long* __restrict__ acc)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.nb || i == 0 || i + 1 == P.nb) return;  // the first and last bead have no tangent
    const uint32_t c = i % P.L;
    const uint32_t a = c == 0 ? i : i - 1, b = c + 1 == P.L ? i : i + 1;
    const float4 pa = pos[a], pb = pos[b], r = pos[i];
    float3 d = make_float3(pb.x - pa.x, pb.y - pa.y, pb.z - pa.z);
    if (min_image) nw::min_image(P, d);
    const float q = d.x * d.x + d.y * d.y;
    const int gx = (int)floor(((double)r.x - G.ox) / G.cs), gy = (int)floor(((double)r.y - G.oy) / G.cs);
    if (gx < 0 || gy < 0 || gx >= (int)G.nx || gy >= (int)G.ny) return;  // not reached: the grid spans the beads
    long long* cell = acc + 2ull * ((size_t)gx * G.ny + gy);
    if (!(q > 0.f)) return;
    const float c2 = (d.x * d.x - d.y * d.y) / q, s2 = (2.f * d.x * d.y) / q;  // cos 2a, sin 2a
    atomicAdd((unsigned long long*)cell, (unsigned long long)llrint((double)c2 * kFix));
    atomicAdd((unsigned long long*)(cell + 1), (unsigned long long)llrint((double)s2 * kFix));
}

// Director angle of a cell: the nematic tensor's, as the representative the
// reference's eigenvector gives: [-pi/4, 3pi/4), -pi/2 for an exactly
// vertical director (diagonal tensor), 0 for an empty or isotropic cell.
__device__ __forceinline__ float cell_theta(const long long* acc, const DefectGrid& G, uint32_t x, uint32_t y)
{
    const long long* c = acc + 2ull * ((size_t)x * G.ny + y);
    const long long C = c[0], S = c[1];
    if (S == 0) return C < 0 ? -0.5f * kPi : 0.f;
    float t = 0.5f * atan2f((float)((double)S / kFix), (float)((double)C / kFix));
    if (t < -0.25f * kPi) t += kPi;
    return t;
}

// rotation from t1 to t2 of a headless director (analysis/find_defects.py:62-68)
__device__ __forceinline__ float theta_step(float t1, float t2)
{
    float d = t2 - t1;
    if (d >= 0.5f * kPi) d -= kPi;
    else if (d <= -0.5f * kPi) d += kPi;
    return d;
}

__global__ void __launch_bounds__(256) defect_circuit_kernel(DefectGrid G, const long long* __restrict__ acc,
                                                             uint32_t* __restrict__ marks, uint32_t* __restrict__ nmarks,
                                                             uint32_t cap)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= G.nx * G.ny) return;
    const uint32_t x = k / G.ny, y = k - x * G.ny;
    if (x < 1 || y < 1 || x + 1 >= G.nx || y + 1 >= G.ny) return;
    // the ring of the 8 neighbours from (+1, 0) round to (+1, 0), counter-clockwise
    const int rx[9] = {1, 1, 0, -1, -1, -1, 0, 1, 1}, ry[9] = {0, 1, 1, 1, 0, -1, -1, -1, 0};
    float t1 = cell_theta(acc, G, x + 1, y), total = 0.f;
#pragma unroll
    for (int s = 1; s < 9; ++s) {
        const float t2 = cell_theta(acc, G, x + rx[s], y + ry[s]);
        total += theta_step(t1, t2);
        t1 = t2;
    }
    const float delta = kPi / 16.f;
    if (total > kPi - delta || total < -kPi + delta) {
        const uint32_t slot = atomicAdd(nmarks, 1u);
        if (slot < cap) marks[slot] = (k << 1) | (total > 0.f ? 1u : 0u);
    }
}

// Touching marked cells (8-neighbourhood, no wrap) of one sign merged; each
// cluster labelled by its first cell in x-major order, the fixed point of the
// reference's lowest-neighbour relabelling (analysis/find_defects.py:126-160).
// cells are sorted by x * ny + y, so each cell's earlier neighbours, (x-1, y-1..y+1)
// and (x, y-1), are found with a pointer that only moves forward.
struct Cluster {
    double sx, sy;  // sums of the member cells' x and y indices
    uint32_t n;     // member cells
};

void cluster(const std::vector<uint32_t>& cells, uint32_t ny, std::vector<Cluster>& out)
{
    const size_t n = cells.size();
    std::vector<uint32_t> parent(n);
    for (size_t a = 0; a < n; ++a) parent[a] = (uint32_t)a;
    auto find = [&](uint32_t a) {
        while (parent[a] != a) a = parent[a] = parent[parent[a]];
        return a;
    };
    auto unite = [&](uint32_t a, uint32_t b) {
        const uint32_t ra = find(a), rb = find(b);
        if (ra != rb) parent[std::max(ra, rb)] = std::min(ra, rb);
    };
    size_t p = 0;  // first cell at or after (x-1, y-1)
    for (size_t a = 0; a < n; ++a) {
        const uint32_t k = cells[a], x = k / ny, y = k % ny;
        if (a > 0 && y > 0 && cells[a - 1] == k - 1) unite((uint32_t)a, (uint32_t)(a - 1));
        if (x == 0) continue;
        const uint32_t lo = (x - 1) * ny + (y > 0 ? y - 1 : 0), hi = (x - 1) * ny + std::min(y + 1, ny - 1);
        while (p < a && cells[p] < lo) ++p;
        for (size_t q = p; q < a && cells[q] <= hi; ++q) unite((uint32_t)a, (uint32_t)q);
    }
    // clusters in order of their first cell (each root is its cluster's lowest
    // index); member index sums in cell order, exact in double
    std::vector<int> slot(n, -1);
    for (size_t a = 0; a < n; ++a) {
        const uint32_t r = find((uint32_t)a);
        if (slot[r] < 0) {
            slot[r] = (int)out.size();
            out.push_back(Cluster{0.0, 0.0, 0u});
        }
        Cluster& c = out[slot[r]];
        c.sx += (double)(cells[a] / ny);
        c.sy += (double)(cells[a] % ny);
        ++c.n;
    }
}

}  // namespace

// ---- the sampling search (analysis/defects.py) ------------------------------

constexpr int kSectors = 8;

// Unit tangent of bead i in float64 (analysis/afa/utils.py:35-49): zero for
// the first and the last bead of the system and for coincident neighbours.
__device__ __forceinline__ void tangent64(const nw::DevParams& P, const float4* __restrict__ pos, uint32_t i,
                                          bool min_image, double& tx, double& ty)
{
    tx = ty = 0.0;
    if (i == 0 || i + 1 >= P.nb) return;
    const uint32_t c = i % P.L;
    const uint32_t a = c == 0 ? i : i - 1, b = c + 1 == P.L ? i : i + 1;
    const float4 pa = pos[a], pb = pos[b];
    double dx, dy, dz;
    if (min_image) {
        float3 d = make_float3(pb.x - pa.x, pb.y - pa.y, pb.z - pa.z);
        nw::min_image(P, d);
        dx = d.x, dy = d.y, dz = d.z;
    } else {
        dx = (double)pb.x - (double)pa.x, dy = (double)pb.y - (double)pa.y, dz = (double)pb.z - (double)pa.z;
    }
    const double nrm = sqrt(dx * dx + dy * dy + dz * dz);
    if (nrm > 0.0) tx = dx / nrm, ty = dy / nrm;
}

// One block per sample point: per-sector sums of the tangents of the beads
// within the radius, combined in a fixed order, then the winding value.
__global__ void __launch_bounds__(256) sample_defect_kernel(const nw::DevParams P, const float4* __restrict__ pos,
                                                            const uint32_t* __restrict__ beads, double r2,
                                                            bool min_image, int32_t* __restrict__ winding)
{
    __shared__ double s_x[kSectors][8], s_y[kSectors][8];
    __shared__ uint32_t s_n[kSectors][8];
    const uint32_t centre = beads[blockIdx.x];
    const float4 c4 = pos[centre];
    const double cx = c4.x, cy = c4.y;
    const double w = 2.0 * 3.141592653589793 / 8.0;  // BIN_EDGES[8] of analysis/afa/utils.py:8-11
    double sx[kSectors], sy[kSectors];
    uint32_t sn[kSectors];
#pragma unroll
    for (int k = 0; k < kSectors; ++k) sx[k] = sy[k] = 0.0, sn[k] = 0u;
    for (uint32_t i = threadIdx.x; i < P.nb; i += blockDim.x) {
        const float4 r = pos[i];
        const double dx = (double)r.x - cx, dy = (double)r.y - cy;
        if (!(dx * dx + dy * dy <= r2)) continue;
        const double ang = atan2(dy, dx);
        int bin = -1;  // np.digitize(angle, edges) - 1: edges at or below the angle, less one
#pragma unroll
        for (int k = 0; k < kSectors; ++k) bin += (double)(k - 4) * w <= ang ? 1 : 0;
        double tx, ty;
        tangent64(P, pos, i, min_image, tx, ty);
#pragma unroll
        for (int k = 0; k < kSectors; ++k)
            if (k == bin) sx[k] += tx, sy[k] += ty, ++sn[k];
    }
    const uint32_t lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < kSectors; ++k) {
#pragma unroll
        for (int o = 16; o; o >>= 1) {
            sx[k] += __shfl_down_sync(0xffffffffu, sx[k], o);
            sy[k] += __shfl_down_sync(0xffffffffu, sy[k], o);
            sn[k] += __shfl_down_sync(0xffffffffu, sn[k], o);
        }
        if (lane == 0) s_x[k][wid] = sx[k], s_y[k][wid] = sy[k], s_n[k][wid] = sn[k];
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    double ang[kSectors];
    int top = -1;
    for (int k = 0; k < kSectors; ++k) {
        double X = 0.0, Y = 0.0;
        uint32_t n = 0;
        for (uint32_t q = 0; q < (blockDim.x >> 5); ++q) X += s_x[k][q], Y += s_y[k][q], n += s_n[k][q];
        ang[k] = n ? atan2(Y / (double)n, X / (double)n) : 0.0;  // compute_director_angle of the mean
        if (n) top = k;
    }
    // winding_number(director_angles, pi) = round(sum(diff(angles / pi)))
    double sum = 0.0;
    for (int k = 0; k < top; ++k) sum += ang[k + 1] / 3.141592653589793 - ang[k] / 3.141592653589793;
    winding[blockIdx.x] = (int32_t)rint(sum);
}

// Fixed workspace: 8 words of bounds and counters, then the marked cells.
constexpr uint32_t kMarkCap = 1u << 16;  // marked cells reported (defects are rare)
constexpr uint32_t kMarkFirst = 4096;    // marked cells copied back with the count

extern "C" nw_status nw_find_defects(nw_system* s, float cell_size, uint32_t flags, NwDefect* out, int max_out,
                                     int* n_out)
{
    if (!s || !n_out || max_out < 0 || (max_out > 0 && !out)) return NW_ERR_INVALID;
    if (!(cell_size > 0.f) || !std::isfinite(cell_size) || (flags & ~NW_DEFECT_MIN_IMAGE)) return NW_ERR_INVALID;
    if (s->cfg.dim >= 3) return NW_ERR_UNSUPPORTED;
    *n_out = 0;
    if (s->nb == 0) return NW_OK;
    const float4* pos = s->B.pos2[s->lists ? (uint32_t)((s->step + 1ull) & 1ull) : 0u];
    auto fail = [](cudaError_t e) {
        cudaGetLastError();
        return e == cudaErrorMemoryAllocation ? NW_ERR_NOMEM : NW_ERR_CUDA;
    };
    cudaError_t e = cudaSuccess;
    if (!s->defect_fixed) e = cudaMalloc(&s->defect_fixed, 32 + (size_t)kMarkCap * 4);
    if (e == cudaSuccess && !s->defect_host) e = cudaMallocHost(&s->defect_host, 32 + (size_t)kMarkFirst * 4);
    if (e != cudaSuccess) return fail(e);
    uint32_t* box = (uint32_t*)s->defect_fixed;  // lo x, lo y, hi x, hi y, marked cells
    uint32_t* marks = box + 8;
    uint32_t* h = s->defect_host;
    e = cudaMemsetAsync(box, 0xff, 8, s->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(box + 2, 0, 12, s->stream);
    if (e == cudaSuccess) {
        defect_bounds_kernel<<<std::min<uint32_t>((s->nb + 255) / 256, 2 * 152), 256, 0, s->stream>>>(pos, s->nb, box);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(h, box, 16, cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return fail(e);
    const double lx = ord_val(h[0]), ly = ord_val(h[1]), hx = ord_val(h[2]), hy = ord_val(h[3]);
    const double cs = (double)cell_size;
    const double fx = std::ceil((hx - lx + 0.0001) / cs), fy = std::ceil((hy - ly + 0.0001) / cs);
    if (!std::isfinite(lx + ly + hx + hy) || !(fx * fy < (double)(1u << 30)))
        return NW_ERR_INVALID;  // non-finite positions or a grid too fine for the beads' extent
    const DefectGrid G{(uint32_t)fx, (uint32_t)fy, cs, lx, ly};
    const size_t ncell = (size_t)G.nx * G.ny, acc_bytes = ncell * 2 * sizeof(long long);
    if (acc_bytes > s->defect_acc_bytes) {
        cudaFree(s->defect_acc);
        s->defect_acc = nullptr;
        s->defect_acc_bytes = 0;
        e = cudaMalloc(&s->defect_acc, acc_bytes);
        if (e != cudaSuccess) return fail(e);
        s->defect_acc_bytes = acc_bytes;
    }
    long long* acc = (long long*)s->defect_acc;
    const nw::DevParams P = nw::make_dev_params(s->cfg, s->cfg.dt);
    e = cudaMemsetAsync(acc, 0, acc_bytes, s->stream);
    if (e == cudaSuccess) {
        defect_bin_kernel<<<(s->nb + 255) / 256, 256, 0, s->stream>>>(P, pos, G, (flags & NW_DEFECT_MIN_IMAGE) != 0,
                                                                       acc);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        defect_circuit_kernel<<<(uint32_t)((ncell + 255) / 256), 256, 0, s->stream>>>(G, acc, marks, box + 4,
                                                                                       kMarkCap);
        e = cudaGetLastError();
    }
    // the count and the first marked cells in one copy (box + 4 .. marks + kMarkFirst)
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(h + 4, box + 4, 16 + (size_t)kMarkFirst * 4, cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return fail(e);
    const uint32_t nm = h[4];
    if (nm > kMarkCap) return NW_ERR_CELL_OVERFLOW;
    std::vector<uint32_t> m(h + 8, h + 8 + std::min(nm, kMarkFirst));
    if (nm > kMarkFirst) {
        m.resize(nm);
        e = cudaMemcpy(m.data() + kMarkFirst, marks + kMarkFirst, (size_t)(nm - kMarkFirst) * 4,
                       cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return fail(e);
    }
    std::sort(m.begin(), m.end());  // x-major cell order
    const double ox = G.ox + 0.0 + G.cs / 2.0, oy = G.oy + 0.0 + G.cs / 2.0;  // the first cell's centre
    int n = 0;
    for (int sign = 1; sign >= 0; --sign) {
        std::vector<uint32_t> cells;
        for (uint32_t v : m)
            if ((v & 1u) == (uint32_t)sign) cells.push_back(v >> 1);
        std::vector<Cluster> clusters;
        cluster(cells, G.ny, clusters);
        for (const Cluster& cl : clusters) {
            const double mx = cl.sx / (double)cl.n, my = cl.sy / (double)cl.n;
            if (n < max_out) out[n] = NwDefect{mx * G.cs + ox, my * G.cs + oy, sign ? 0.5f : -0.5f, cl.n};
            ++n;
        }
    }
    *n_out = n;
    return NW_OK;
}

extern "C" nw_status nw_sample_defects(nw_system* s, const uint32_t* beads, int n_points, float radius,
                                       uint32_t flags, int32_t* winding)
{
    if (!s || n_points < 0 || (n_points > 0 && (!beads || !winding))) return NW_ERR_INVALID;
    if (!(radius >= 0.f) || !std::isfinite(radius) || (flags & ~NW_DEFECT_MIN_IMAGE)) return NW_ERR_INVALID;
    if (s->cfg.dim >= 3) return NW_ERR_UNSUPPORTED;
    if (n_points == 0) return NW_OK;
    for (int k = 0; k < n_points; ++k)
        if (beads[k] >= s->nb) return NW_ERR_INVALID;
    const float4* pos = s->B.pos2[s->lists ? (uint32_t)((s->step + 1ull) & 1ull) : 0u];
    // the system's defect workspace holds up to kMarkCap / 2 points; more take their own
    uint32_t* d_beads = nullptr;
    int32_t* d_w = nullptr;
    const bool own = (uint32_t)n_points > kMarkCap / 2u;
    cudaError_t e = cudaSuccess;
    if (!own && !s->defect_fixed) e = cudaMalloc(&s->defect_fixed, 32 + (size_t)kMarkCap * 4);
    if (e == cudaSuccess && !own) {
        d_beads = (uint32_t*)s->defect_fixed + 8;
        d_w = (int32_t*)(d_beads + n_points);
    }
    if (e == cudaSuccess && own) e = cudaMalloc(&d_beads, (size_t)n_points * 4);
    if (e == cudaSuccess && own) e = cudaMalloc(&d_w, (size_t)n_points * 4);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_beads, beads, (size_t)n_points * 4, cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess) {
        const nw::DevParams P = nw::make_dev_params(s->cfg, s->cfg.dt);
        const double r = (double)radius;
        sample_defect_kernel<<<(uint32_t)n_points, 256, 0, s->stream>>>(P, pos, d_beads, r * r,
                                                                         (flags & NW_DEFECT_MIN_IMAGE) != 0, d_w);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(winding, d_w, (size_t)n_points * 4, cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (own) {
        cudaFree(d_beads);
        cudaFree(d_w);
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        return e == cudaErrorMemoryAllocation ? NW_ERR_NOMEM : NW_ERR_CUDA;
    }
    return NW_OK;
}
