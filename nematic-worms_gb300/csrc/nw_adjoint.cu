// nw_adjoint.cu — differentiable rollout of the WCA worm step
// (include/nwgb_adjoint.h): a forward pass on frozen neighbour lists with a
// fixed noise realisation, checkpoints every `segment` steps, and a
// hand-written adjoint of the force and integrate steps.
//
// Step of update m (mass 1, the engine's ordering):
//   v_m = v_{m-1} + dt/2 (F_{m-1} + F_{m-2})
//   r_m = wrap(r_{m-1} + dt v_m + dt^2/2 F_{m-1})
//   F_m = -gamma v_m + sigma xi_m + Fc(r_m; theta)
// with Fc = eps F_lj + k_bend F_bend + k_bond F_bond + F_act F_drive (each
// term linear in its parameter).  Adjoint of update m, from the adjoints
// (lr, lv, lF, lFo) of (r_m, v_m, F_m, F_{m-1}):
//   lr~ = lr + Jc^T lF          lv~ = lv - gamma lF + dt lr~
//   lF(m-1) = lFo + dt^2/2 lr~ + dt/2 lv~,   lFo(m-1) = dt/2 lv~
//   lr(m-1) = lr~,  lv(m-1) = lv~,  dL/dtheta_k += lF . F_k(r_m)
// Jc^T lF: the LJ, bond and bending terms are conservative (symmetric
// Jacobian), so Jc^T lF = Jc lF is taken as a directional derivative (dual
// numbers for the bending triple, closed forms for the central pair laws);
// the drive F_i = F_act (r_{i+1} - r_i)/|.| is not, and is transposed
// explicitly.  Every bead's output has one writer; per-block parameter
// gradients are summed in a fixed order, so runs are bit-reproducible.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/nwgb_adjoint.h"
#include "nw_engine.h"

using namespace nw;

namespace {

template <class T>
struct V3 {
    T x, y, z;
};
template <class T>
__host__ __device__ __forceinline__ V3<T> v3(T x, T y, T z)
{
    return V3<T>{x, y, z};
}
template <class T>
__device__ __forceinline__ V3<T> operator+(V3<T> a, V3<T> b)
{
    return v3(a.x + b.x, a.y + b.y, a.z + b.z);
}
template <class T>
__device__ __forceinline__ V3<T> operator-(V3<T> a, V3<T> b)
{
    return v3(a.x - b.x, a.y - b.y, a.z - b.z);
}
template <class T, class S>
__device__ __forceinline__ V3<T> operator*(S s, V3<T> a)
{
    return v3(T(s) * a.x, T(s) * a.y, T(s) * a.z);
}
template <class T>
__device__ __forceinline__ T dot(V3<T> a, V3<T> b)
{
    return a.x * b.x + a.y * b.y + a.z * b.z;
}

// Dual number a + b e (e^2 = 0): value and directional derivative.
template <class T>
struct D {
    T v, d;
};
template <class T>
__device__ __forceinline__ D<T> operator+(D<T> a, D<T> b)
{
    return D<T>{a.v + b.v, a.d + b.d};
}
template <class T>
__device__ __forceinline__ D<T> operator-(D<T> a, D<T> b)
{
    return D<T>{a.v - b.v, a.d - b.d};
}
template <class T>
__device__ __forceinline__ D<T> operator-(D<T> a)
{
    return D<T>{-a.v, -a.d};
}
template <class T>
__device__ __forceinline__ D<T> operator*(D<T> a, D<T> b)
{
    return D<T>{a.v * b.v, a.v * b.d + a.d * b.v};
}
template <class T>
__device__ __forceinline__ D<T> operator/(D<T> a, D<T> b)
{
    const T q = a.v / b.v;
    return D<T>{q, (a.d - q * b.d) / b.v};
}
template <class T>
__device__ __forceinline__ D<T> dsqrt(D<T> a)
{
    const T s = sqrt(a.v);
    return D<T>{s, a.d / (T(2) * s)};
}
template <class T>
__device__ __forceinline__ T dsqrt(T a)
{
    return sqrt(a);
}
template <class T>
__device__ __forceinline__ T val(T a)
{
    return a;
}
template <class T>
__device__ __forceinline__ T val(D<T> a)
{
    return a.v;
}
template <class T>
__device__ __forceinline__ void shift(T& a, T s)
{
    a -= s;
}
template <class T>
__device__ __forceinline__ void shift(D<T>& a, T s)
{
    a.v -= s;
}

template <class T>
struct Vec4;
template <>
struct Vec4<float> {
    using type = float4;
};
template <>
struct Vec4<double> {
    using type = double4;
};

template <class T>
struct AdjParams {
    uint32_t nb, L, R, N;
    int32_t dim;
    T box[3], half[3], origin[3];
    T two_s6, lj_unit, rc2, rl2;
    int32_t exclude;
    T r0, gamma, sigma, dt;
    int32_t langevin_on;
    T eps, kbend, kbond, fact;
    unsigned long long seed;
    uint32_t lg[3], lcells, cap, ncap;
    T linv[3];
};

template <class T>
__device__ __forceinline__ V3<T> ld3(const typename Vec4<T>::type* a, uint32_t i)
{
    const typename Vec4<T>::type q = a[i];
    return v3<T>(q.x, q.y, q.z);
}
template <class T>
__device__ __forceinline__ void st3(typename Vec4<T>::type* a, uint32_t i, V3<T> x)
{
    typename Vec4<T>::type q;
    q.x = x.x;
    q.y = x.y;
    q.z = x.z;
    q.w = T(0);
    a[i] = q;
}

// Minimum image on the value (the shift is piecewise constant: no tangent).
template <class T, class S>
__device__ __forceinline__ void min_img(const AdjParams<T>& P, S& x, S& y, S& z)
{
    S* c[3] = {&x, &y, &z};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const T v = val(*c[a]);
        if (v > P.half[a]) shift(*c[a], P.box[a]);
        else if (v < -P.half[a]) shift(*c[a], -P.box[a]);
    }
}

// Bending triple with unit stiffness in scalar type S (T or D<T>):
// A = 1/(d_ij d_jk), F_i = -A (b - a (a.b)/|a|^2), F_k = -A (b (a.b)/|b|^2 - a),
// F_j = -F_i - F_k with a = r_j - r_i, b = r_k - r_j.
template <class S>
struct Tri {
    S fi[3], fj[3], fk[3];
};
template <class T, class S>
__device__ __forceinline__ Tri<S> bend_unit(const AdjParams<T>& P, const S ri[3], const S rj[3], const S rk[3])
{
    S a[3], b[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        a[q] = rj[q] - ri[q];
        b[q] = rk[q] - rj[q];
    }
    min_img(P, a[0], a[1], a[2]);
    min_img(P, b[0], b[1], b[2]);
    const S qa = a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
    const S qb = b[0] * b[0] + b[1] * b[1] + b[2] * b[2];
    const S dd = a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
    const S one = qa / qa;  // 1 with a zero tangent in either scalar type
    const S A = one / dsqrt(qa * qb);
    const S sa = dd / qa, sb = dd / qb;
    Tri<S> t;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        t.fi[q] = -(A * (b[q] - a[q] * sa));
        t.fk[q] = -(A * (b[q] * sb - a[q]));
        t.fj[q] = -t.fi[q] - t.fk[q];
    }
    return t;
}

template <class T>
__device__ __forceinline__ V3<T> noise(const AdjParams<T>& P, uint32_t rep, uint32_t li, unsigned long long step)
{
    const unsigned long long key = P.seed + rep;
    const uint4 x = philox4x32_10(make_uint4(li, (uint32_t)step, (uint32_t)(step >> 32), kRngLangevin), (uint32_t)key,
                                  (uint32_t)(key >> 32));
    T z2 = T(0);
    T s, c;
    const T r0 = sqrt(T(-2) * log(T(u01(x.x))));
    sincospi(T(2) * T(u01(x.y)), &s, &c);
    const T z0 = r0 * c, z1 = r0 * s;
    if (P.dim >= 3) {
        const T r1 = sqrt(T(-2) * log(T(u01(x.z))));
        T s1, c1;
        sincospi(T(2) * T(u01(x.w)), &s1, &c1);
        z2 = r1 * c1;
    }
    return v3<T>(P.sigma * z0, P.sigma * z1, P.sigma * z2);
}

// ---- list build -------------------------------------------------------------------

template <class T>
__device__ __forceinline__ uint32_t lcell(const AdjParams<T>& P, V3<T> r, uint32_t rep)
{
    const T x[3] = {r.x, r.y, r.z};
    uint32_t c[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const int G = (int)P.lg[a];
        int g = G == 1 ? 0 : (int)floor((x[a] - P.origin[a]) * P.linv[a]);
        g %= G;
        if (g < 0) g += G;
        c[a] = (uint32_t)g;
    }
    return rep * P.lcells + (c[2] * P.lg[1] + c[1]) * P.lg[0] + c[0];
}

template <class T>
__global__ void __launch_bounds__(256) adj_bin_kernel(const AdjParams<T> P, const typename Vec4<T>::type* __restrict__ r,
                                                      uint32_t* __restrict__ cnt, uint32_t* __restrict__ slot,
                                                      uint32_t* __restrict__ err)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.N) return;
    const uint32_t h = lcell(P, ld3<T>(r, i), i / P.nb);
    const uint32_t k = atomicAdd(cnt + h, 1u);
    if (k < P.cap) slot[(size_t)h * P.cap + k] = i;
    else atomicOr(err, (uint32_t)NW_EFLAG_CELL_OVERFLOW);
}

// Neighbours of bead i within lj_rcut + skin (not itself, not same-filament
// pairs within lj_exclude), ascending: the order does not depend on the
// order the cells were filled in.
template <class T>
__global__ void __launch_bounds__(256) adj_list_kernel(const AdjParams<T> P, const typename Vec4<T>::type* __restrict__ r,
                                                       const uint32_t* __restrict__ cnt,
                                                       const uint32_t* __restrict__ slot, uint32_t* __restrict__ nbr,
                                                       uint32_t* __restrict__ nnb, uint32_t* __restrict__ err)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.N) return;
    const uint32_t rep = i / P.nb, li = i - rep * P.nb;
    const uint32_t fbase = i - li % P.L;
    const V3<T> ri = ld3<T>(r, i);
    const uint32_t own = lcell(P, ri, rep) - rep * P.lcells;
    uint32_t c[3];
    c[0] = own % P.lg[0];
    c[1] = (own / P.lg[0]) % P.lg[1];
    c[2] = own / (P.lg[0] * P.lg[1]);
    uint32_t k = 0;
    // offsets -1, 0, +1 per axis; with fewer than three cells the repeats are skipped
    for (int dz = -1; dz <= 1; ++dz) {
        if (P.lg[2] < 3 && dz != 0 && (P.lg[2] == 1 || dz == 1)) continue;
        const uint32_t z = (c[2] + P.lg[2] + dz) % P.lg[2];
        for (int dy = -1; dy <= 1; ++dy) {
            if (P.lg[1] < 3 && dy != 0 && (P.lg[1] == 1 || dy == 1)) continue;
            const uint32_t y = (c[1] + P.lg[1] + dy) % P.lg[1];
            for (int dx = -1; dx <= 1; ++dx) {
                if (P.lg[0] < 3 && dx != 0 && (P.lg[0] == 1 || dx == 1)) continue;
                const uint32_t x = (c[0] + P.lg[0] + dx) % P.lg[0];
                const uint32_t h = rep * P.lcells + (z * P.lg[1] + y) * P.lg[0] + x;
                uint32_t m = cnt[h];
                if (m > P.cap) m = P.cap;
                for (uint32_t q = 0; q < m; ++q) {
                    const uint32_t j = slot[(size_t)h * P.cap + q];
                    if (j == i) continue;
                    const int d = (int)j - (int)i;
                    if (d <= P.exclude && d >= -P.exclude && j - fbase < P.L) continue;
                    V3<T> dr = ld3<T>(r, j) - ri;
                    min_img(P, dr.x, dr.y, dr.z);
                    if (dot(dr, dr) > P.rl2) continue;
                    // insertion into the ascending list
                    if (k < P.ncap) {
                        uint32_t p = k;
                        while (p > 0 && nbr[(size_t)(p - 1) * P.N + i] > j) {
                            nbr[(size_t)p * P.N + i] = nbr[(size_t)(p - 1) * P.N + i];
                            --p;
                        }
                        nbr[(size_t)p * P.N + i] = j;
                    }
                    ++k;
                }
            }
        }
    }
    nnb[i] = k < P.ncap ? k : P.ncap;
    if (k > P.ncap) atomicOr(err, (uint32_t)NW_EFLAG_NEIGHBOR_OVERFLOW);
}

// ---- forward ---------------------------------------------------------------------

template <class T>
__global__ void __launch_bounds__(256) adj_integrate_kernel(const AdjParams<T> P, typename Vec4<T>::type* __restrict__ r,
                                                            typename Vec4<T>::type* __restrict__ v,
                                                            typename Vec4<T>::type* __restrict__ F,
                                                            typename Vec4<T>::type* __restrict__ Fo,
                                                            typename Vec4<T>::type* __restrict__ traj)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.N) return;
    const V3<T> f = ld3<T>(F, i), fo = ld3<T>(Fo, i);
    const V3<T> vn = ld3<T>(v, i) + (T(0.5) * P.dt) * (f + fo);
    V3<T> rn = ld3<T>(r, i) + P.dt * vn + (T(0.5) * P.dt * P.dt) * f;
    T* c[3] = {&rn.x, &rn.y, &rn.z};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (*c[a] < P.origin[a]) *c[a] += P.box[a];
        else if (*c[a] > P.origin[a] + P.box[a]) *c[a] -= P.box[a];
    }
    st3<T>(v, i, vn);
    st3<T>(r, i, rn);
    st3<T>(Fo, i, f);
    if (traj) st3<T>(traj, i, rn);
}

template <class T>
__device__ __forceinline__ T lj_fm_unit(const AdjParams<T>& P, T q)
{
    const T iq = T(1) / q;
    const T iq4 = iq * iq * iq * iq;
    return P.lj_unit * (P.two_s6 * iq4 * iq * iq * iq - iq4);
}

template <class T>
__global__ void __launch_bounds__(256) adj_force_kernel(const AdjParams<T> P, const typename Vec4<T>::type* __restrict__ r,
                                                        const typename Vec4<T>::type* __restrict__ v,
                                                        typename Vec4<T>::type* __restrict__ F,
                                                        const uint32_t* __restrict__ nbr,
                                                        const uint32_t* __restrict__ nnb, unsigned long long step)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.N) return;
    const uint32_t rep = i / P.nb, li = i - rep * P.nb, c = li % P.L;
    const V3<T> ri = ld3<T>(r, i);
    V3<T> f = v3<T>(0, 0, 0);
    if (P.langevin_on) f = noise(P, rep, li, step) - P.gamma * ld3<T>(v, i);
    // bending, in the engine's triple order (first bead c-2, c-1, c)
    for (int p = (int)c - 2; p <= (int)c; ++p) {
        if (p < 0 || (uint32_t)p + 2 >= P.L) continue;
        const uint32_t b0 = i - c + (uint32_t)p;
        T a[3][3];
        for (int s = 0; s < 3; ++s) {
            const V3<T> x = ld3<T>(r, b0 + s);
            a[s][0] = x.x;
            a[s][1] = x.y;
            a[s][2] = x.z;
        }
        const Tri<T> t = bend_unit<T, T>(P, a[0], a[1], a[2]);
        const T* g = (uint32_t)p == c ? t.fi : ((uint32_t)p + 1 == c ? t.fj : t.fk);
        f = f + P.kbend * v3<T>(g[0], g[1], g[2]);
    }
    // bonds and drive
    for (int s = -1; s <= 1; s += 2) {
        if ((s < 0 && c == 0) || (s > 0 && c + 1 >= P.L)) continue;
        V3<T> dr = ld3<T>(r, i + s) - ri;
        min_img(P, dr.x, dr.y, dr.z);
        const T d = sqrt(dot(dr, dr));
        f = f + (P.kbond * (T(1) - P.r0 / d)) * dr;
        if (s > 0) f = f + (P.fact / d) * dr;
    }
    // LJ over the frozen list
    const uint32_t k = nnb[i];
    for (uint32_t m = 0; m < k; ++m) {
        const uint32_t j = nbr[(size_t)m * P.N + i];
        V3<T> dr = ld3<T>(r, j) - ri;
        min_img(P, dr.x, dr.y, dr.z);
        const T q = dot(dr, dr);
        if (q > P.rc2) continue;
        f = f - (P.eps * lj_fm_unit(P, q)) * dr;
    }
    st3<T>(F, i, f);
}

// ---- adjoint ---------------------------------------------------------------------

__device__ __forceinline__ double warp_sum_d(double x)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    return x;
}

template <class T>
__global__ void __launch_bounds__(256) adj_step_kernel(const AdjParams<T> P, const typename Vec4<T>::type* __restrict__ r,
                                                       const uint32_t* __restrict__ nbr,
                                                       const uint32_t* __restrict__ nnb,
                                                       typename Vec4<T>::type* __restrict__ lr,
                                                       typename Vec4<T>::type* __restrict__ lv,
                                                       const typename Vec4<T>::type* __restrict__ lF_in,
                                                       typename Vec4<T>::type* __restrict__ lF_out,
                                                       typename Vec4<T>::type* __restrict__ lFo,
                                                       double* __restrict__ gacc)
{
    __shared__ double s_g[8][4];
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    double g[4] = {0.0, 0.0, 0.0, 0.0};  // eps, k_bend, k_bond, F_act
    if (i < P.N) {
        const uint32_t rep = i / P.nb, li = i - rep * P.nb, c = li % P.L;
        const V3<T> ri = ld3<T>(r, i);
        const V3<T> lfi = ld3<T>(lF_in, i);
        V3<T> jt = v3<T>(0, 0, 0);
        // bending: directional derivative of the unit triple forces along lF
        for (int p = (int)c - 2; p <= (int)c; ++p) {
            if (p < 0 || (uint32_t)p + 2 >= P.L) continue;
            const uint32_t b0 = i - c + (uint32_t)p;
            D<T> a[3][3];
            for (int s = 0; s < 3; ++s) {
                const V3<T> x = ld3<T>(r, b0 + s), t = ld3<T>(lF_in, b0 + s);
                a[s][0] = D<T>{x.x, t.x};
                a[s][1] = D<T>{x.y, t.y};
                a[s][2] = D<T>{x.z, t.z};
            }
            const Tri<D<T>> t = bend_unit<T, D<T>>(P, a[0], a[1], a[2]);
            const D<T>* q = (uint32_t)p == c ? t.fi : ((uint32_t)p + 1 == c ? t.fj : t.fk);
            g[1] += (double)(lfi.x * q[0].v + lfi.y * q[1].v + lfi.z * q[2].v);
            jt = jt + P.kbend * v3<T>(q[0].d, q[1].d, q[2].d);
        }
        // bonds (central: phi(q) dr with phi = k (1 - r0 / sqrt q)) and the drive
        for (int s = -1; s <= 1; s += 2) {
            if ((s < 0 && c == 0) || (s > 0 && c + 1 >= P.L)) continue;
            V3<T> dr = ld3<T>(r, i + s) - ri;
            min_img(P, dr.x, dr.y, dr.z);
            const T q = dot(dr, dr), d = sqrt(q);
            const V3<T> del = ld3<T>(lF_in, i + s) - lfi;
            const T phi = T(1) - P.r0 / d, dphi = T(0.5) * P.r0 / (q * d);
            g[2] += (double)(phi * dot(lfi, dr));
            jt = jt + P.kbond * (phi * del + (dphi * T(2) * dot(dr, del)) * dr);
            if (s > 0) {
                // own drive F_i = F_act dr / d: d/dr_i = -A, A l = (l - dr (dr . l) / d^2) / d
                g[3] += (double)(dot(lfi, dr) / d);
                jt = jt - (P.fact / d) * (lfi - (dot(dr, lfi) / q) * dr);
            }
        }
        if (c >= 1) {
            // the previous bead's drive depends on r_i with d/dr_i = +A
            V3<T> dr = ri - ld3<T>(r, i - 1);
            min_img(P, dr.x, dr.y, dr.z);
            const T q = dot(dr, dr), d = sqrt(q);
            const V3<T> lp = ld3<T>(lF_in, i - 1);
            jt = jt + (P.fact / d) * (lp - (dot(dr, lp) / q) * dr);
        }
        // LJ over the frozen list: F_i = -eps fm(q) dr, fm' from q
        const uint32_t k = nnb[i];
        for (uint32_t m = 0; m < k; ++m) {
            const uint32_t j = nbr[(size_t)m * P.N + i];
            V3<T> dr = ld3<T>(r, j) - ri;
            min_img(P, dr.x, dr.y, dr.z);
            const T q = dot(dr, dr);
            if (q > P.rc2) continue;
            const T iq = T(1) / q;
            const T iq4 = iq * iq * iq * iq;
            const T fm = P.lj_unit * (P.two_s6 * iq4 * iq * iq * iq - iq4);
            const T dfm = P.lj_unit * (T(-7) * P.two_s6 * iq4 * iq4 + T(4) * iq4 * iq);
            const V3<T> del = ld3<T>(lF_in, j) - lfi;
            g[0] += (double)(-fm * dot(lfi, dr));
            jt = jt - P.eps * ((dfm * T(2) * dot(dr, del)) * dr + fm * del);
        }
        const V3<T> lrt = ld3<T>(lr, i) + jt;
        V3<T> lvt = ld3<T>(lv, i);
        if (P.langevin_on) lvt = lvt - P.gamma * lfi;
        lvt = lvt + P.dt * lrt;
        const V3<T> lfn = ld3<T>(lFo, i) + (T(0.5) * P.dt * P.dt) * lrt + (T(0.5) * P.dt) * lvt;
        st3<T>(lF_out, i, lfn);
        st3<T>(lFo, i, (T(0.5) * P.dt) * lvt);
        st3<T>(lr, i, lrt);
        st3<T>(lv, i, lvt);
    }
    // per-block parameter gradient, one writer per block: a fixed summation order
    const uint32_t lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const double x = warp_sum_d(g[q]);
        if (lane == 0) s_g[w][q] = x;
    }
    __syncthreads();
    if (threadIdx.x < 4) {
        double x = 0.0;
        for (uint32_t k = 0; k < blockDim.x / 32u; ++k) x += s_g[k][threadIdx.x];
        gacc[blockIdx.x * 4u + threadIdx.x] += x;
    }
}

// ---- conversions -------------------------------------------------------------------

template <class T>
__global__ void from_f4_kernel(const float4* __restrict__ a, typename Vec4<T>::type* __restrict__ b, uint32_t n)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) st3<T>(b, i, v3<T>(a[i].x, a[i].y, a[i].z));
}

template <class T>
__global__ void to_f4_kernel(const typename Vec4<T>::type* __restrict__ a, float4* __restrict__ b,
                             const float4* __restrict__ wsrc, uint32_t n)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const V3<T> x = ld3<T>(a, i);
        b[i] = make_float4((float)x.x, (float)x.y, (float)x.z, wsrc ? wsrc[i].w : 0.f);
    }
}

// xyz of the state in double (x, y, z, 0) quadruples, at either precision
template <class T>
__global__ void to_d4_kernel(const typename Vec4<T>::type* __restrict__ a, double* __restrict__ b, uint32_t n)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const V3<T> x = ld3<T>(a, i);
        b[4 * (size_t)i] = (double)x.x;
        b[4 * (size_t)i + 1] = (double)x.y;
        b[4 * (size_t)i + 2] = (double)x.z;
        b[4 * (size_t)i + 3] = 0.0;
    }
}

uint32_t nblocks(uint32_t n) { return (n + 255u) / 256u; }

}  // namespace

struct nw_adjoint {
    NwConfig cfg;
    int R = 0, horizon = 0, seg = 0, prec = 32;
    uint32_t nb = 0, N = 0, nseg = 0;
    cudaStream_t own = nullptr, stream = nullptr;
    size_t elem = 16;  // bytes of one stored vector
    void *r = nullptr, *v = nullptr, *F = nullptr, *Fo = nullptr;
    void *r0 = nullptr, *v0 = nullptr;
    float4* w_pos = nullptr;  // w components of the initial positions (radius) and velocities (mass)
    float4* w_vel = nullptr;
    void* ck = nullptr;    // checkpoints: [nseg][4][N]
    void* traj = nullptr;  // positions of one segment: [seg][N]
    void *lr = nullptr, *lv = nullptr, *lF[2] = {nullptr, nullptr}, *lFo = nullptr;
    uint32_t *cnt = nullptr, *slot = nullptr, *nbr = nullptr, *nnb = nullptr, *err = nullptr;
    double* gacc = nullptr;
    std::vector<void*> allocs;
    double theta[4] = {0, 0, 0, 0};
    bool have_forward = false;
    float fwd_ms = 0.f, bwd_ms = 0.f;
    uint32_t lg[3] = {1, 1, 1}, lcells = 1, cap = 16, ncap = 32;
};

namespace {

template <class T>
AdjParams<T> adj_params(const nw_adjoint* a, const double th[4])
{
    const NwConfig& c = a->cfg;
    AdjParams<T> P;
    std::memset(&P, 0, sizeof(P));
    P.nb = a->nb;
    P.L = c.filament_size;
    P.R = (uint32_t)a->R;
    P.N = a->N;
    P.dim = c.dim;
    for (int k = 0; k < 3; ++k) {
        P.box[k] = (T)c.box[k];
        P.half[k] = (T)c.box[k] / T(2);
        P.origin[k] = (T)c.origin[k];
        P.lg[k] = a->lg[k];
        P.linv[k] = (T)a->lg[k] / (T)c.box[k];
    }
    const double s6 = std::pow((double)c.lj_sigma, 6.0);
    P.two_s6 = (T)(2.0 * s6);
    P.lj_unit = (T)(24.0 * s6);
    P.rc2 = (T)((double)c.lj_rcut * (double)c.lj_rcut);
    const double skin = c.neighbor_skin > 0.0f ? c.neighbor_skin : 0.3 * c.lj_sigma;
    P.rl2 = (T)(((double)c.lj_rcut + skin) * ((double)c.lj_rcut + skin));
    P.exclude = c.lj_exclude;
    P.r0 = (T)c.bond_r0;
    P.gamma = (T)c.gamma;
    double s2 = 2.0 * (double)c.gamma * (double)c.kT;
    if (c.noise_dt_scaling) s2 /= (double)c.dt;
    P.sigma = (T)std::sqrt(s2);
    P.dt = (T)c.dt;
    P.langevin_on = 1;
    P.eps = (T)th[0];
    P.kbend = (T)th[1];
    P.kbond = (T)th[2];
    P.fact = (T)th[3];
    P.seed = c.seed;
    P.lcells = a->lcells;
    P.cap = a->cap;
    P.ncap = a->ncap;
    return P;
}

void* at(void* base, size_t index, const nw_adjoint* a)
{
    return static_cast<char*>(base) + index * (size_t)a->N * a->elem;
}

template <class T>
cudaError_t build_lists(nw_adjoint* a, const AdjParams<T>& P, const void* r)
{
    using V = typename Vec4<T>::type;
    cudaError_t e = cudaMemsetAsync(a->cnt, 0, (size_t)a->R * a->lcells * 4, a->stream);
    if (e != cudaSuccess) return e;
    adj_bin_kernel<T><<<nblocks(a->N), 256, 0, a->stream>>>(P, static_cast<const V*>(r), a->cnt, a->slot, a->err);
    adj_list_kernel<T><<<nblocks(a->N), 256, 0, a->stream>>>(P, static_cast<const V*>(r), a->cnt, a->slot, a->nbr,
                                                            a->nnb, a->err);
    return cudaGetLastError();
}

// Updates [m0, m1) (1-based update m uses noise counter m - 1) from the
// current state; positions after each update go to traj[m - m0] if asked.
template <class T>
cudaError_t run_updates(nw_adjoint* a, const AdjParams<T>& P, int m0, int m1, bool keep)
{
    using V = typename Vec4<T>::type;
    for (int m = m0; m < m1; ++m) {
        V* tr = keep ? static_cast<V*>(at(a->traj, (size_t)(m - m0), a)) : nullptr;
        adj_integrate_kernel<T><<<nblocks(a->N), 256, 0, a->stream>>>(P, static_cast<V*>(a->r), static_cast<V*>(a->v),
                                                                      static_cast<V*>(a->F), static_cast<V*>(a->Fo), tr);
        adj_force_kernel<T><<<nblocks(a->N), 256, 0, a->stream>>>(P, static_cast<const V*>(a->r),
                                                                  static_cast<const V*>(a->v), static_cast<V*>(a->F),
                                                                  a->nbr, a->nnb, (unsigned long long)(m - 1));
    }
    return cudaGetLastError();
}

cudaError_t save_state(nw_adjoint* a, uint32_t s, bool to_ck)
{
    void* st[4] = {a->r, a->v, a->F, a->Fo};
    const size_t bytes = (size_t)a->N * a->elem;
    for (int k = 0; k < 4; ++k) {
        void* c = at(a->ck, (size_t)s * 4 + k, a);
        cudaError_t e = to_ck ? cudaMemcpyAsync(c, st[k], bytes, cudaMemcpyDeviceToDevice, a->stream)
                              : cudaMemcpyAsync(st[k], c, bytes, cudaMemcpyDeviceToDevice, a->stream);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

nw_status st_of(cudaError_t e)
{
    if (e == cudaSuccess) return NW_OK;
    cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? NW_ERR_NOMEM : NW_ERR_CUDA;
}

nw_status check_err(nw_adjoint* a)
{
    uint32_t f = 0;
    cudaError_t e = cudaMemcpyAsync(&f, a->err, 4, cudaMemcpyDeviceToHost, a->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(a->stream);
    if (e != cudaSuccess) return st_of(e);
    if (f) {
        cudaMemsetAsync(a->err, 0, 4, a->stream);
        cudaStreamSynchronize(a->stream);
        return NW_ERR_CELL_OVERFLOW;
    }
    return NW_OK;
}

template <class T>
nw_status forward_t(nw_adjoint* a, const double th[4], float* pos_out, float* vel_out)
{
    using V = typename Vec4<T>::type;
    const AdjParams<T> P = adj_params<T>(a, th);
    const size_t bytes = (size_t)a->N * a->elem;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, a->stream);
    cudaError_t e = cudaMemcpyAsync(a->r, a->r0, bytes, cudaMemcpyDeviceToDevice, a->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(a->v, a->v0, bytes, cudaMemcpyDeviceToDevice, a->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(a->F, 0, bytes, a->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(a->Fo, 0, bytes, a->stream);
    for (uint32_t s = 0; s < a->nseg && e == cudaSuccess; ++s) {
        e = save_state(a, s, true);
        if (e == cudaSuccess) e = build_lists<T>(a, P, a->r);
        const int m0 = (int)s * a->seg + 1, m1 = std::min(a->horizon, (int)(s + 1) * a->seg) + 1;
        if (e == cudaSuccess) e = run_updates<T>(a, P, m0, m1, false);
    }
    cudaEventRecord(e1, a->stream);
    if (e == cudaSuccess && pos_out)
        to_f4_kernel<T><<<nblocks(a->N), 256, 0, a->stream>>>(static_cast<const V*>(a->r), (float4*)pos_out, a->w_pos,
                                                              a->N);
    if (e == cudaSuccess && vel_out)
        to_f4_kernel<T><<<nblocks(a->N), 256, 0, a->stream>>>(static_cast<const V*>(a->v), (float4*)vel_out, a->w_vel,
                                                              a->N);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(a->stream);
    if (e == cudaSuccess) cudaEventElapsedTime(&a->fwd_ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) return st_of(e);
    const nw_status st = check_err(a);
    if (st != NW_OK) return st;
    std::memcpy(a->theta, th, sizeof(a->theta));
    a->have_forward = true;
    return NW_OK;
}

template <class T>
nw_status backward_t(nw_adjoint* a, const float* gpos, const float* gvel, double out[4])
{
    using V = typename Vec4<T>::type;
    const AdjParams<T> P = adj_params<T>(a, a->theta);
    const size_t bytes = (size_t)a->N * a->elem;
    const uint32_t nbk = nblocks(a->N);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, a->stream);
    from_f4_kernel<T><<<nbk, 256, 0, a->stream>>>((const float4*)gpos, static_cast<V*>(a->lr), a->N);
    from_f4_kernel<T><<<nbk, 256, 0, a->stream>>>((const float4*)gvel, static_cast<V*>(a->lv), a->N);
    cudaError_t e = cudaMemsetAsync(a->lF[0], 0, bytes, a->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(a->lFo, 0, bytes, a->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(a->gacc, 0, (size_t)nbk * 4 * sizeof(double), a->stream);
    uint32_t cur = 0;
    for (int s = (int)a->nseg - 1; s >= 0 && e == cudaSuccess; --s) {
        e = save_state(a, (uint32_t)s, false);
        if (e == cudaSuccess) e = build_lists<T>(a, P, a->r);
        const int m0 = s * a->seg + 1, m1 = std::min(a->horizon, (s + 1) * a->seg) + 1;
        if (e == cudaSuccess) e = run_updates<T>(a, P, m0, m1, true);
        for (int m = m1 - 1; m >= m0 && e == cudaSuccess; --m) {
            adj_step_kernel<T><<<nbk, 256, 0, a->stream>>>(
                P, static_cast<const V*>(at(a->traj, (size_t)(m - m0), a)), a->nbr, a->nnb, static_cast<V*>(a->lr),
                static_cast<V*>(a->lv), static_cast<const V*>(a->lF[cur]), static_cast<V*>(a->lF[cur ^ 1u]),
                static_cast<V*>(a->lFo), a->gacc);
            cur ^= 1u;
            e = cudaGetLastError();
        }
    }
    cudaEventRecord(e1, a->stream);
    std::vector<double> g((size_t)nbk * 4);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(g.data(), a->gacc, g.size() * sizeof(double), cudaMemcpyDeviceToHost, a->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(a->stream);
    if (e == cudaSuccess) cudaEventElapsedTime(&a->bwd_ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) return st_of(e);
    const nw_status st = check_err(a);
    if (st != NW_OK) return st;
    for (int q = 0; q < 4; ++q) {
        double x = 0.0;
        for (uint32_t b = 0; b < nbk; ++b) x += g[(size_t)b * 4 + q];
        out[q] = x;
    }
    return NW_OK;
}

}  // namespace

extern "C" {

nw_status nw_adj_create(const NwConfig* cfg, int n_replicas, int horizon, int segment, int precision,
                        nw_adjoint** out)
{
    if (!out) return NW_ERR_INVALID;
    *out = nullptr;
    if (!cfg || n_replicas <= 0 || horizon <= 0 || segment <= 0 || (precision != 32 && precision != 64))
        return NW_ERR_INVALID;
    nw_status st = nw_config_validate(cfg);
    if (st != NW_OK) return st;
    if (cfg->model != NW_MODEL_WCA_WORMS || cfg->srd_enabled || cfg->reverse_probability > 0.0f)
        return NW_ERR_UNSUPPORTED;
    for (int k = 0; k < 3; ++k)
        if (cfg->boundary[k] != NW_PERIODIC) return NW_ERR_UNSUPPORTED;
    const uint64_t nb = (uint64_t)cfg->num_filaments * cfg->filament_size;
    if (nb == 0 || nb * (uint64_t)n_replicas >= (1ull << 31)) return NW_ERR_INVALID;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return NW_ERR_NO_DEVICE;
    }
    nw_adjoint* a = new nw_adjoint();
    a->cfg = *cfg;
    a->R = n_replicas;
    a->horizon = horizon;
    a->seg = segment;
    a->prec = precision;
    a->nb = (uint32_t)nb;
    a->N = (uint32_t)(nb * (uint64_t)n_replicas);
    a->nseg = (uint32_t)((horizon + segment - 1) / segment);
    a->elem = precision == 64 ? 32 : 16;
    const double skin = cfg->neighbor_skin > 0.0f ? cfg->neighbor_skin : 0.3 * cfg->lj_sigma;
    const double rl = (double)cfg->lj_rcut + skin;
    a->lcells = 1;
    for (int k = 0; k < 3; ++k) {
        uint32_t G = 1;
        if (cfg->grid[k] > 1) {
            const double g = std::floor((double)cfg->box[k] / (rl * 1.0001));
            G = g >= 1.0 ? (uint32_t)g : 1u;
        }
        a->lg[k] = G;
        a->lcells *= G;
    }
    a->ncap = cfg->neighbor_capacity ? cfg->neighbor_capacity : 32u;
    a->cap = 16;
    // a blocking stream: the rollout's own work is ordered with the legacy
    // default stream, on which callers such as torch produce the upstream
    // gradients it reads (a non-blocking stream could read them unfinished)
    if (cudaStreamCreateWithFlags(&a->own, cudaStreamDefault) != cudaSuccess) {
        delete a;
        return NW_ERR_CUDA;
    }
    a->stream = a->own;
    auto A = [&](void** p, size_t bytes) {
        if (st != NW_OK) return;
        if (cudaMalloc(p, bytes ? bytes : 16) != cudaSuccess) {
            cudaGetLastError();
            st = NW_ERR_NOMEM;
            return;
        }
        a->allocs.push_back(*p);
    };
    const size_t vb = (size_t)a->N * a->elem;
    A(&a->r, vb);
    A(&a->v, vb);
    A(&a->F, vb);
    A(&a->Fo, vb);
    A(&a->r0, vb);
    A(&a->v0, vb);
    A((void**)&a->w_pos, (size_t)a->N * 16);
    A((void**)&a->w_vel, (size_t)a->N * 16);
    A(&a->ck, vb * 4 * a->nseg);
    A(&a->traj, vb * (size_t)segment);
    A(&a->lr, vb);
    A(&a->lv, vb);
    A(&a->lF[0], vb);
    A(&a->lF[1], vb);
    A(&a->lFo, vb);
    A((void**)&a->cnt, (size_t)a->R * a->lcells * 4);
    A((void**)&a->slot, (size_t)a->R * a->lcells * a->cap * 4);
    A((void**)&a->nbr, (size_t)a->N * a->ncap * 4);
    A((void**)&a->nnb, (size_t)a->N * 4);
    A((void**)&a->err, 16);
    A((void**)&a->gacc, (size_t)nblocks(a->N) * 4 * sizeof(double));
    if (st == NW_OK) st = st_of(cudaMemset(a->err, 0, 16));
    if (st != NW_OK) {
        nw_adj_destroy(a);
        return st;
    }
    *out = a;
    return NW_OK;
}

nw_status nw_adj_destroy(nw_adjoint* a)
{
    if (!a) return NW_ERR_INVALID;
    cudaStreamSynchronize(a->stream);
    for (void* p : a->allocs) cudaFree(p);
    if (a->own) cudaStreamDestroy(a->own);
    delete a;
    return NW_OK;
}

nw_status nw_adj_set_stream(nw_adjoint* a, void* stream)
{
    if (!a) return NW_ERR_INVALID;
    cudaStreamSynchronize(a->stream);
    a->stream = stream ? (cudaStream_t)stream : a->own;
    return NW_OK;
}

nw_status nw_adj_set_state(nw_adjoint* a, const float* d_pos, const float* d_vel)
{
    if (!a || !d_pos || !d_vel) return NW_ERR_INVALID;
    const uint32_t nbk = nblocks(a->N);
    if (a->prec == 64) {
        from_f4_kernel<double><<<nbk, 256, 0, a->stream>>>((const float4*)d_pos, (double4*)a->r0, a->N);
        from_f4_kernel<double><<<nbk, 256, 0, a->stream>>>((const float4*)d_vel, (double4*)a->v0, a->N);
    } else {
        from_f4_kernel<float><<<nbk, 256, 0, a->stream>>>((const float4*)d_pos, (float4*)a->r0, a->N);
        from_f4_kernel<float><<<nbk, 256, 0, a->stream>>>((const float4*)d_vel, (float4*)a->v0, a->N);
    }
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(a->w_pos, d_pos, (size_t)a->N * 16, cudaMemcpyDeviceToDevice, a->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(a->w_vel, d_vel, (size_t)a->N * 16, cudaMemcpyDeviceToDevice, a->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(a->stream);
    a->have_forward = false;
    return st_of(e);
}

nw_status nw_adj_forward(nw_adjoint* a, const double theta[4], float* d_pos_out, float* d_vel_out)
{
    if (!a || !theta) return NW_ERR_INVALID;
    for (int q = 0; q < 4; ++q)
        if (!std::isfinite(theta[q])) return NW_ERR_INVALID;
    return a->prec == 64 ? forward_t<double>(a, theta, d_pos_out, d_vel_out)
                         : forward_t<float>(a, theta, d_pos_out, d_vel_out);
}

nw_status nw_adj_final_state_f64(nw_adjoint* a, double* d_pos_out, double* d_vel_out)
{
    if (!a || !a->have_forward) return NW_ERR_INVALID;
    cudaError_t e = cudaSuccess;
    if (a->prec == 64) {
        using V = typename Vec4<double>::type;
        if (d_pos_out) to_d4_kernel<double><<<nblocks(a->N), 256, 0, a->stream>>>(static_cast<const V*>(a->r), d_pos_out, a->N);
        if (d_vel_out) to_d4_kernel<double><<<nblocks(a->N), 256, 0, a->stream>>>(static_cast<const V*>(a->v), d_vel_out, a->N);
    } else {
        using V = typename Vec4<float>::type;
        if (d_pos_out) to_d4_kernel<float><<<nblocks(a->N), 256, 0, a->stream>>>(static_cast<const V*>(a->r), d_pos_out, a->N);
        if (d_vel_out) to_d4_kernel<float><<<nblocks(a->N), 256, 0, a->stream>>>(static_cast<const V*>(a->v), d_vel_out, a->N);
    }
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(a->stream);
    return e == cudaSuccess ? NW_OK : st_of(e);
}

nw_status nw_adj_backward(nw_adjoint* a, const float* d_grad_pos, const float* d_grad_vel, double grad_theta[4])
{
    if (!a || !d_grad_pos || !d_grad_vel || !grad_theta) return NW_ERR_INVALID;
    if (!a->have_forward) return NW_ERR_INVALID;
    return a->prec == 64 ? backward_t<double>(a, d_grad_pos, d_grad_vel, grad_theta)
                         : backward_t<float>(a, d_grad_pos, d_grad_vel, grad_theta);
}

nw_status nw_adj_timings(const nw_adjoint* a, float* forward_ms, float* backward_ms)
{
    if (!a) return NW_ERR_INVALID;
    if (forward_ms) *forward_ms = a->fwd_ms;
    if (backward_ms) *backward_ms = a->bwd_ms;
    return NW_OK;
}

}  // extern "C"
