// nw_observables.cu — observables of the current state on the device
// (include/nwgb.h, "observables"): order parameters, temperatures and the
// mean-square displacement in one pass over the beads and solvent, the
// velocity correlation of sampled bead pairs by distance, and the histogram
// of SRD cell temperatures.
//
// Sums are deterministic: per-block partial sums in double, reduced by one
// block in block order (nw_observe, nw_velocity_correlation), or integer
// atomics on fixed-point values (the SRD cell sums: the same integers
// whatever the thread order).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "nw_engine.h"
#include "nw_system.h"

namespace {

constexpr uint32_t kObsThreads = 256;
constexpr uint32_t kObsBlocks = 4 * 152;
constexpr uint32_t kObsSums = 16;
constexpr double kFix = 4294967296.0;  // 2^32: fixed point of the SRD cell sums

// sums of the bead pass, in this order
enum {
    S_TXX, S_TYY, S_TZZ, S_TXY, S_TXZ, S_TYZ,  // sum of t t
    S_TX, S_TY, S_TZ,                          // sum of t
    S_C2, S_S2,                                // sum of cos 2a, sin 2a (xy tangent angle)
    S_BEAD_KE2,                                // sum of m |v|^2 over beads
    S_MSD,                                     // sum of |r_unwrapped - r_ref|^2
    S_SOLV_KE2,                                // sum of m |v|^2 over the solvent
    S_NT,                                      // beads with a tangent
    S_PAD
};

struct ObsArgs {
    const float4* pos;
    const float4* vel;
    const float4* spos;
    const float4* svel;
    uint32_t nb, ns, L, dim;
    float box[3];
    int periodic[3];
    int min_image;
    // mean-square displacement bookkeeping (msd on): reference and last seen
    // positions, periodic images crossed since the reference
    const float4* msd_ref;
    float4* msd_last;
    int4* msd_img;
    int msd;
};

__device__ __forceinline__ float3 sub3(float4 a, float4 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }

__device__ __forceinline__ void wrap_min(const ObsArgs& A, float3& d)
{
    if (A.periodic[0]) d.x -= A.box[0] * rintf(d.x / A.box[0]);
    if (A.periodic[1]) d.y -= A.box[1] * rintf(d.y / A.box[1]);
    if (A.periodic[2]) d.z -= A.box[2] * rintf(d.z / A.box[2]);
}

// Tangent of bead i as the reference's analysis takes it
// (analysis/afa/utils.py:35-49): unit(r[i+1] - r[i-1]), r[i] in place of
// r[i-1] at a filament's head and of r[i+1] at its tail; the first and the
// last bead of the system get none (the analysis centres its windows on
// beads 1 .. n-2).  Raw differences, or the minimum image.
__device__ __forceinline__ bool tangent(const ObsArgs& A, uint32_t i, float3& t)
{
    if (i == 0 || i + 1 >= A.nb) return false;
    const uint32_t c = i % A.L;
    const uint32_t a = c == 0 ? i : i - 1, b = c == A.L - 1 ? i : i + 1;
    float3 d = sub3(A.pos[b], A.pos[a]);
    if (A.min_image) wrap_min(A, d);
    const double n = sqrt((double)d.x * d.x + (double)d.y * d.y + (double)d.z * d.z);
    if (!(n > 0.0)) return false;
    t = make_float3((float)(d.x / n), (float)(d.y / n), (float)(d.z / n));
    return true;
}

__device__ __forceinline__ double block_sum(double x, double* sh)
{
#pragma unroll
    for (int o = 16; o; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    const uint32_t w = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    __syncthreads();
    if (lane == 0) sh[w] = x;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (uint32_t k = 0; k < blockDim.x / 32u; ++k) s += sh[k];
    return s;
}

__global__ void __launch_bounds__(kObsThreads) observe_kernel(const ObsArgs A, double* __restrict__ partial)
{
    __shared__ double sh[kObsThreads / 32];
    double acc[S_PAD];
#pragma unroll
    for (int k = 0; k < S_PAD; ++k) acc[k] = 0.0;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < A.nb; i += stride) {
        float3 t;
        if (tangent(A, i, t)) {
            const double x = t.x, y = t.y, z = t.z;
            acc[S_TXX] += x * x, acc[S_TYY] += y * y, acc[S_TZZ] += z * z;
            acc[S_TXY] += x * y, acc[S_TXZ] += x * z, acc[S_TYZ] += y * z;
            acc[S_TX] += x, acc[S_TY] += y, acc[S_TZ] += z;
            const double q = x * x + y * y;
            if (q > 0.0) {
                acc[S_C2] += (x * x - y * y) / q;
                acc[S_S2] += 2.0 * x * y / q;
            }
            acc[S_NT] += 1.0;
        }
        const float4 v = A.vel[i];
        acc[S_BEAD_KE2] += (double)v.w * ((double)v.x * v.x + (double)v.y * v.y + (A.dim >= 3 ? (double)v.z * v.z : 0.0));
        if (A.msd) {
            const float4 r = A.pos[i], last = A.msd_last[i];
            int4 im = A.msd_img[i];
            const float d[3] = {r.x - last.x, r.y - last.y, r.z - last.z};
            int* ip[3] = {&im.x, &im.y, &im.z};
            for (int a = 0; a < 3; ++a)
                if (A.periodic[a]) {
                    if (d[a] > 0.5f * A.box[a]) *ip[a] -= 1;
                    else if (d[a] < -0.5f * A.box[a]) *ip[a] += 1;
                }
            A.msd_img[i] = im;
            A.msd_last[i] = r;
            const float4 r0 = A.msd_ref[i];
            const double ux = (double)r.x + (double)im.x * A.box[0] - r0.x;
            const double uy = (double)r.y + (double)im.y * A.box[1] - r0.y;
            const double uz = (double)r.z + (double)im.z * A.box[2] - r0.z;
            acc[S_MSD] += ux * ux + uy * uy + uz * uz;
        }
    }
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < A.ns; i += stride) {
        const float4 v = A.svel[i];
        acc[S_SOLV_KE2] += (double)v.w * ((double)v.x * v.x + (double)v.y * v.y + (A.dim >= 3 ? (double)v.z * v.z : 0.0));
    }
    for (int k = 0; k < S_PAD; ++k) {
        const double s = block_sum(acc[k], sh);
        if (threadIdx.x == 0) partial[(size_t)blockIdx.x * kObsSums + k] = s;
    }
}

// partial sums of the blocks, added in block order by one block
__global__ void __launch_bounds__(kObsSums) reduce_partials_kernel(const double* __restrict__ partial, uint32_t nblocks,
                                                                  uint32_t width, double* __restrict__ out)
{
    for (uint32_t k = threadIdx.x; k < width; k += blockDim.x) {
        double s = 0.0;
        for (uint32_t b = 0; b < nblocks; ++b) s += partial[(size_t)b * width + k];
        out[k] = s;
    }
}

__global__ void msd_reset_kernel(const float4* __restrict__ pos, uint32_t nb, float4* __restrict__ ref,
                                 float4* __restrict__ last, int4* __restrict__ img)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nb) {
        ref[i] = pos[i];
        last[i] = pos[i];
        img[i] = make_int4(0, 0, 0, 0);
    }
}

// ---- velocity correlation by distance --------------------------------------------

// Quadratic B-spline weights of distance d on `bins` bins of width w (the
// weights nwgb.observables.bin_weights gives): centre c = floor(x + 1/2),
// x = d / w - 1/2, t = x - c; weights 0.5 (0.5 - t)^2, 0.75 - t^2,
// 0.5 (0.5 + t)^2 on bins c - 1, c, c + 1 (outside 0 .. bins-1 dropped).
template <int MAXB>
__global__ void __launch_bounds__(32) vcorr_kernel(const ObsArgs A, const uint32_t* __restrict__ pi,
                                                            const uint32_t* __restrict__ pj, uint32_t n, double w,
                                                            uint32_t bins, double* __restrict__ partial,
                                                            uint32_t* __restrict__ bad)
{
    __shared__ double s_sum[MAXB], s_wt[MAXB];
    for (uint32_t k = threadIdx.x; k < bins; k += blockDim.x) s_sum[k] = s_wt[k] = 0.0;
    __syncthreads();
    // blocks of one warp: each chunk of 32 pairs is added to the block's sums
    // by lane 0, lane by lane, so the sums do not depend on scheduling
    const uint32_t warps = blockDim.x / 32u, lane = threadIdx.x & 31u;
    const uint32_t gw = blockIdx.x * warps + (threadIdx.x >> 5), nw = gridDim.x * warps;
    for (uint32_t base = gw * 32u; base < n; base += nw * 32u) {
        const uint32_t p = base + lane;
        int c = -100;
        double wt[3] = {0.0, 0.0, 0.0}, dot = 0.0;
        if (p < n) {
            const uint32_t i = pi[p], j = pj[p];
            if (i >= A.nb || j >= A.nb) {
                atomicOr(bad, 1u);
            } else {
                float3 d = sub3(A.pos[j], A.pos[i]);
                wrap_min(A, d);
                const double dist = sqrt((double)d.x * d.x + (double)d.y * d.y + (double)d.z * d.z);
                const double x = dist / w - 0.5, cc = floor(x + 0.5), t = x - cc;
                c = (int)cc;
                wt[0] = 0.5 * (0.5 - t) * (0.5 - t);
                wt[1] = 0.75 - t * t;
                wt[2] = 0.5 * (0.5 + t) * (0.5 + t);
                const float4 vi = A.vel[i], vj = A.vel[j];
                dot = (double)vi.x * vj.x + (double)vi.y * vj.y + (double)vi.z * vj.z;
            }
        }
        // lanes in order: the warp's contributions enter the block sums lane by lane
        for (uint32_t l = 0; l < 32u; ++l) {
            const int cl = __shfl_sync(0xffffffffu, c, l);
            const double dl = __shfl_sync(0xffffffffu, dot, l);
            for (int q = 0; q < 3; ++q) {
                const double wl = __shfl_sync(0xffffffffu, wt[q], l);
                const int b = cl - 1 + q;
                if (lane == 0 && b >= 0 && b < (int)bins && wl != 0.0) {
                    s_sum[b] += wl * dl;
                    s_wt[b] += wl;
                }
            }
        }
        __syncwarp();
    }
    __syncthreads();
    for (uint32_t k = threadIdx.x; k < bins; k += blockDim.x) {
        partial[(size_t)blockIdx.x * 2 * bins + k] = s_sum[k];
        partial[(size_t)blockIdx.x * 2 * bins + bins + k] = s_wt[k];
    }
}

// ---- SRD cell temperatures ---------------------------------------------------------

struct SrdHistArgs {
    uint32_t grid[3], ncells;
    float cell[3], origin[3], box[3], shift[3];
    int periodic[3];
    uint32_t dim;
};

__device__ __forceinline__ long long fix(double x) { return llrint(__dmul_rn(x, kFix)); }

__device__ __forceinline__ int srd_axis(const SrdHistArgs& H, int a, float x)
{
    // position relative to the box after the grid shift, wrapped on periodic axes
    float p = x + H.shift[a] - H.origin[a];
    if (H.periodic[a]) {
        if (p >= H.box[a]) p -= H.box[a];
        else if (p < 0.0f) p += H.box[a];
    }
    int g = (int)floorf(p / H.cell[a]);
    const int G = (int)H.grid[a];
    if (H.periodic[a]) {
        g %= G;
        if (g < 0) g += G;
    } else {
        g = g < 0 ? 0 : (g >= G ? G - 1 : g);
    }
    return g;
}

__global__ void __launch_bounds__(256) srd_cell_sums_kernel(const SrdHistArgs H, const float4* __restrict__ pos,
                                                            const float4* __restrict__ vel, uint32_t n,
                                                            unsigned long long* __restrict__ acc)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 r = pos[i], v = vel[i];
    const int gx = srd_axis(H, 0, r.x), gy = srd_axis(H, 1, r.y);
    const int gz = H.grid[2] > 1u ? srd_axis(H, 2, r.z) : 0;
    const uint32_t c = ((uint32_t)gz * H.grid[1] + (uint32_t)gy) * H.grid[0] + (uint32_t)gx;
    const double m = v.w;
    const double vz = H.dim >= 3 ? (double)v.z : 0.0;
    unsigned long long* a = acc + (size_t)c * 6;
    atomicAdd(a + 0, 1ull);
    atomicAdd(a + 1, (unsigned long long)fix(m));
    atomicAdd(a + 2, (unsigned long long)fix(__dmul_rn(m, v.x)));
    atomicAdd(a + 3, (unsigned long long)fix(__dmul_rn(m, v.y)));
    atomicAdd(a + 4, (unsigned long long)fix(__dmul_rn(m, vz)));
    // separately rounded products and sums (no fused multiply-add), so that
    // a host restatement forms the same integers
    const double q = __dadd_rn(__dadd_rn(__dmul_rn(v.x, v.x), __dmul_rn(v.y, v.y)), __dmul_rn(vz, vz));
    atomicAdd(a + 5, (unsigned long long)fix(__dmul_rn(m, q)));
}

// cell temperature sum m |v - u|^2 / (dim (n - 1)), u the cell's mass-weighted mean velocity
__global__ void __launch_bounds__(256) srd_hist_kernel(const unsigned long long* __restrict__ acc, uint32_t ncells,
                                                       uint32_t dim, double t_max, uint32_t bins,
                                                       unsigned int* __restrict__ counts)
{
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncells) return;
    const unsigned long long* a = acc + (size_t)c * 6;
    const unsigned long long n = a[0];
    if (n < 2) return;
    const double M = (double)(long long)a[1] / kFix;
    const double px = (double)(long long)a[2] / kFix, py = (double)(long long)a[3] / kFix;
    const double pz = (double)(long long)a[4] / kFix, ke2 = (double)(long long)a[5] / kFix;
    const double p2 = __dadd_rn(__dadd_rn(__dmul_rn(px, px), __dmul_rn(py, py)), __dmul_rn(pz, pz));
    const double rel = __dsub_rn(ke2, p2 / M);
    const double T = rel / ((double)dim * (double)(n - 1));
    const double b = floor(T / t_max * (double)bins);
    const uint32_t k = b < 0.0 ? 0u : (b >= (double)bins ? bins : (uint32_t)b);  // bins = overflow
    atomicAdd(counts + k, 1u);
    atomicAdd(counts + bins + 1, 1u);
}

nw_status cuda_st(cudaError_t e)
{
    if (e == cudaSuccess) return NW_OK;
    cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? NW_ERR_NOMEM : NW_ERR_CUDA;
}

ObsArgs obs_args(const nw_system* s, uint32_t flags)
{
    ObsArgs A{};
    const uint32_t cur = s->lists ? (uint32_t)((s->step + 1ull) & 1ull) : 0u;
    A.pos = s->B.pos2[cur];
    A.vel = s->B.vel2[cur];
    A.spos = s->B.spos2[s->scur];
    A.svel = s->B.svel2[s->scur];
    A.nb = s->nb;
    A.ns = s->cfg.srd_enabled ? s->ns : 0u;
    A.L = s->cfg.filament_size ? s->cfg.filament_size : 1u;
    A.dim = s->cfg.dim;
    for (int a = 0; a < 3; ++a) {
        A.box[a] = s->cfg.box[a];
        A.periodic[a] = s->cfg.boundary[a] == NW_PERIODIC;
    }
    A.min_image = (flags & NW_OBS_MIN_IMAGE) != 0;
    return A;
}

cudaError_t ensure(void** p, size_t* have, size_t bytes)
{
    if (*p && *have >= bytes) return cudaSuccess;
    cudaFree(*p);
    *p = nullptr;
    *have = 0;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e == cudaSuccess) *have = bytes;
    return e;
}

// largest eigenvalue of a symmetric 3 x 3 matrix (trigonometric solution of
// the characteristic cubic; O. K. Smith, CACM 4(4):168, 1961)
double sym3_max_eigenvalue(const double q[6])
{
    const double a = q[0], b = q[1], c = q[2], d = q[3], e = q[4], f = q[5];  // xx yy zz xy xz yz
    const double p1 = d * d + e * e + f * f;
    if (p1 == 0.0) return std::max(a, std::max(b, c));
    const double m = (a + b + c) / 3.0;
    const double p2 = (a - m) * (a - m) + (b - m) * (b - m) + (c - m) * (c - m) + 2.0 * p1;
    const double p = std::sqrt(p2 / 6.0);
    const double B[6] = {(a - m) / p, (b - m) / p, (c - m) / p, d / p, e / p, f / p};
    const double detB = B[0] * (B[1] * B[2] - B[5] * B[5]) - B[3] * (B[3] * B[2] - B[5] * B[4]) +
                        B[4] * (B[3] * B[5] - B[1] * B[4]);
    double r = detB / 2.0;
    r = r < -1.0 ? -1.0 : (r > 1.0 ? 1.0 : r);
    const double phi = std::acos(r) / 3.0;
    return m + 2.0 * p * std::cos(phi);
}

}  // namespace

extern "C" {

nw_status nw_observe_reset(nw_system* s)
{
    if (!s) return NW_ERR_INVALID;
    const size_t nb = s->nb ? s->nb : 1u;
    cudaError_t e = ensure(&s->obs_msd, &s->obs_msd_bytes, nb * (16 + 16 + 16));
    if (e != cudaSuccess) return cuda_st(e);
    float4* ref = static_cast<float4*>(s->obs_msd);
    float4* last = ref + nb;
    int4* img = reinterpret_cast<int4*>(last + nb);
    const ObsArgs A = obs_args(s, 0u);
    if (s->nb) msd_reset_kernel<<<(s->nb + 255u) / 256u, 256, 0, s->stream>>>(A.pos, s->nb, ref, last, img);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e == cudaSuccess) s->obs_msd_on = true;
    return cuda_st(e);
}

nw_status nw_observe(nw_system* s, uint32_t flags, NwObservables* out)
{
    if (!s || !out) return NW_ERR_INVALID;
    ObsArgs A = obs_args(s, flags);
    const size_t nb = s->nb ? s->nb : 1u;
    if ((flags & NW_OBS_MSD) && !s->obs_msd_on) return NW_ERR_INVALID;
    if (flags & NW_OBS_MSD) {
        A.msd = 1;
        A.msd_ref = static_cast<const float4*>(s->obs_msd);
        A.msd_last = static_cast<float4*>(s->obs_msd) + nb;
        A.msd_img = reinterpret_cast<int4*>(static_cast<float4*>(s->obs_msd) + 2 * nb);
    }
    const size_t need = (size_t)kObsBlocks * kObsSums * 8 + kObsSums * 8;
    cudaError_t e = ensure(&s->obs_ws, &s->obs_ws_bytes, need);
    if (e != cudaSuccess) return cuda_st(e);
    double* partial = static_cast<double*>(s->obs_ws);
    double* sums = partial + (size_t)kObsBlocks * kObsSums;
    observe_kernel<<<kObsBlocks, kObsThreads, 0, s->stream>>>(A, partial);
    reduce_partials_kernel<<<1, kObsSums, 0, s->stream>>>(partial, kObsBlocks, kObsSums, sums);
    double h[kObsSums];
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(h, sums, sizeof(h), cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return cuda_st(e);
    std::memset(out, 0, sizeof(*out));
    const double n = (double)s->nb;
    out->n_beads = s->nb;
    out->n_tangents = (uint32_t)h[S_NT];
    const double dim = (double)s->cfg.dim;
    if (s->nb) {
        // Q = 1.5 <t t> - I / 2 over all beads (those without a tangent count as zero)
        double q[6];
        for (int k = 0; k < 6; ++k) q[k] = 1.5 * h[S_TXX + k] / n - (k < 3 ? 0.5 : 0.0);
        out->s_q3 = sym3_max_eigenvalue(q);
        const double nt = h[S_NT] > 0.0 ? h[S_NT] : 1.0;
        out->s_2d = std::sqrt(h[S_C2] * h[S_C2] + h[S_S2] * h[S_S2]) / nt;
        out->polar = std::sqrt(h[S_TX] * h[S_TX] + h[S_TY] * h[S_TY] + h[S_TZ] * h[S_TZ]) / n;
        out->bead_temperature = h[S_BEAD_KE2] / (dim * n);
        out->msd = (flags & NW_OBS_MSD) ? h[S_MSD] / n : 0.0;
    }
    if (A.ns) out->solvent_temperature = h[S_SOLV_KE2] / (dim * (double)A.ns);
    out->n_solvent = A.ns;
    return NW_OK;
}

nw_status nw_velocity_correlation(nw_system* s, const uint32_t* d_i, const uint32_t* d_j, uint32_t n_pairs,
                                  float r_max, uint32_t bins, double* sum_dot, double* sum_weight)
{
    if (!s || (!d_i && n_pairs) || (!d_j && n_pairs) || !sum_dot || !sum_weight || bins == 0 || bins > 128 ||
        !(r_max > 0.0f))
        return NW_ERR_INVALID;
    const ObsArgs A = obs_args(s, NW_OBS_MIN_IMAGE);
    const uint32_t nblk = std::max(1u, std::min(kObsBlocks, (n_pairs + 31u) / 32u));
    const size_t need = (size_t)nblk * 2 * bins * 8 + 2 * (size_t)bins * 8 + 16;
    cudaError_t e = ensure(&s->obs_ws, &s->obs_ws_bytes, std::max(need, (size_t)kObsBlocks * kObsSums * 8 + kObsSums * 8));
    if (e != cudaSuccess) return cuda_st(e);
    double* partial = static_cast<double*>(s->obs_ws);
    double* sums = partial + (size_t)nblk * 2 * bins;
    uint32_t* bad = reinterpret_cast<uint32_t*>(sums + 2 * bins);
    e = cudaMemsetAsync(bad, 0, 4, s->stream);
    // one warp per block: its lane 0 alone writes the shared sums, in lane order
    if (e == cudaSuccess && n_pairs)
        vcorr_kernel<128><<<nblk, 32, 0, s->stream>>>(A, d_i, d_j, n_pairs, (double)r_max / bins, bins, partial, bad);
    if (e == cudaSuccess && n_pairs) reduce_partials_kernel<<<1, kObsSums, 0, s->stream>>>(partial, nblk, 2 * bins, sums);
    if (e == cudaSuccess) e = cudaGetLastError();
    std::vector<double> h(2 * bins, 0.0);
    uint32_t hb = 0;
    if (e == cudaSuccess && n_pairs) e = cudaMemcpyAsync(h.data(), sums, 2 * bins * 8, cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&hb, bad, 4, cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return cuda_st(e);
    if (hb) return NW_ERR_INVALID;
    std::memcpy(sum_dot, h.data(), bins * 8);
    std::memcpy(sum_weight, h.data() + bins, bins * 8);
    return NW_OK;
}

nw_status nw_srd_temperature_histogram(nw_system* s, const float shift[3], float t_max, uint32_t bins,
                                       uint32_t* counts)
{
    if (!s || !counts || bins == 0 || bins > 4096 || !(t_max > 0.0f) || !s->cfg.srd_enabled) return NW_ERR_INVALID;
    SrdHistArgs H{};
    for (int a = 0; a < 3; ++a) {
        H.grid[a] = s->cfg.srd_grid[a];
        H.cell[a] = s->cfg.srd_cell_size[a];
        H.origin[a] = s->cfg.origin[a];
        H.box[a] = s->cfg.box[a];
        H.shift[a] = shift ? shift[a] : 0.0f;
        H.periodic[a] = s->cfg.boundary[a] == NW_PERIODIC;
    }
    H.ncells = s->srd_ncells;
    H.dim = s->cfg.dim;
    const size_t acc_bytes = (size_t)H.ncells * 6 * 8;
    cudaError_t e = ensure(&s->obs_srd, &s->obs_srd_bytes, acc_bytes + (size_t)(bins + 2) * 4);
    if (e != cudaSuccess) return cuda_st(e);
    unsigned long long* acc = static_cast<unsigned long long*>(s->obs_srd);
    unsigned int* cnt = reinterpret_cast<unsigned int*>(static_cast<char*>(s->obs_srd) + acc_bytes);
    e = cudaMemsetAsync(s->obs_srd, 0, acc_bytes + (size_t)(bins + 2) * 4, s->stream);
    const ObsArgs A = obs_args(s, 0u);
    if (e == cudaSuccess && A.nb)
        srd_cell_sums_kernel<<<(A.nb + 255u) / 256u, 256, 0, s->stream>>>(H, A.pos, A.vel, A.nb, acc);
    if (e == cudaSuccess && A.ns)
        srd_cell_sums_kernel<<<(A.ns + 255u) / 256u, 256, 0, s->stream>>>(H, A.spos, A.svel, A.ns, acc);
    if (e == cudaSuccess)
        srd_hist_kernel<<<(H.ncells + 255u) / 256u, 256, 0, s->stream>>>(acc, H.ncells, H.dim, (double)t_max, bins,
                                                                        cnt);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(counts, cnt, (size_t)(bins + 2) * 4, cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    return cuda_st(e);
}

}  // extern "C"
