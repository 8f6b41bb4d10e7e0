/*
 * nw_oracle_impl.h — precision-generic body of the CPU oracle (TEST
 * INFRASTRUCTURE ONLY).  Included by nw_oracle.c with R = float / double and
 * RS(name) appending the _f32 / _f64 suffix.
 *
 * Each routine restates one reference kernel; the reference file:line it
 * follows is given above it.  FP32 arithmetic keeps the reference's
 * operation order so that FP32 results agree with the device to rounding.
 */

/* lengthPeriodic (simulation/particles_kernel_impl.cuh:279-301): minimum
 * image on periodic axes, single shift, in place; returns |dr|. */
static R RS(length_periodic)(const NwConfig* cfg, R dr[3])
{
    for (int a = 0; a < 3; ++a) {
        if (cfg->boundary[a] != NW_PERIODIC) continue;
        R L = (R)cfg->box[a];
        R Lo2 = L / (R)2;
        if (dr[a] > Lo2) dr[a] -= L;
        else if (dr[a] < -Lo2) dr[a] += L;
    }
    return (R)sqrt((double)(dr[0] * dr[0] + dr[1] * dr[1] + dr[2] * dr[2]));
}

static R RS(dot3)(const R a[3], const R b[3])
{
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

static R RS(rsqrt_len)(R x)
{
    return (R)sqrt((double)x);
}

/* periodicBoundary / dampedWallBoundary / noslipWallBoundary
 * (simulation/particles_kernel_impl.cuh:34-68) in the per-axis order of
 * filament_integrator (:99-134): x, y, then z (z has no no-slip branch). */
static void RS(apply_boundaries)(const NwConfig* cfg, R p[3], R v[3], const R dr[3], R rad)
{
    for (int a = 0; a < 3; ++a) {
        const R L0 = (R)cfg->origin[a];
        const R L = (R)cfg->box[a];
        const int b = cfg->boundary[a];
        if (b == NW_PERIODIC) {
            if (p[a] < L0) p[a] += L;
            else if (p[a] > L + L0) p[a] -= L;
        } else if (b == NW_WALL) {
            const R coef = (R)cfg->boundary_damping;
            if (p[a] < L0 + rad) {
                p[a] = L0 + rad;
                v[a] *= coef;
            } else if (p[a] > (L + L0) - rad) {
                p[a] = (L + L0) - rad;
                v[a] *= coef;
            }
        } else if (b == NW_WALL_NO_SLIP && a < 2) {
            const R N[3] = {(R)(a == 0), (R)(a == 1), (R)0};
            int hit = 0;
            R target = 0;
            if (p[a] < L0 + rad) {
                hit = 1;
                target = L0 + rad;
            } else if (p[a] > (L + L0) - rad) {
                hit = 1;
                target = (L + L0) - rad;
            }
            if (hit) {
                for (int c = 0; c < 3; ++c) p[c] -= dr[c];
                p[a] = target;
                for (int c = 0; c < 3; ++c) v[c] = -v[c] * N[c];
            }
        }
    }
}

/* filament_integrator (simulation/particles_kernel_impl.cuh:71-142). */
void RS(nwo_integrate)(const NwConfig* cfg, R* pos, R* vel, R* force, R* force_old, uint32_t n, R dt)
{
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < (long long)n; ++i) {
        R* P = pos + 4 * i;
        R* V = vel + 4 * i;
        R* F = force + 4 * i;
        R* Fo = force_old + 4 * i;
        R p[3], v[3], f[3], fo[3], dr[3];
        for (int a = 0; a < 3; ++a) {
            p[a] = P[a];
            v[a] = V[a];
            f[a] = F[a];
            fo[a] = Fo[a];
        }
        for (int a = 0; a < 3; ++a) {
            R dv = ((R)0.5 * (f[a] + fo[a])) * dt;
            v[a] += dv;
        }
        for (int a = 0; a < 3; ++a) dr[a] = v[a] * dt + (((R)0.5 * f[a]) * dt) * dt;
        for (int a = 0; a < 3; ++a) p[a] += dr[a];
        RS(apply_boundaries)(cfg, p, v, dr, (R)cfg->radius);
        for (int a = 0; a < 3; ++a) {
            P[a] = p[a];
            V[a] = v[a];
            Fo[a] = f[a];
        }
        F[0] = F[1] = F[2] = F[3] = 0;
    }
}

/* solvent_integrator (simulation/particles_kernel_impl.cuh:145-205): ballistic
 * streaming, boundaries with zero radius. */
void RS(nwo_integrate_solvent)(const NwConfig* cfg, R* pos, R* vel, uint32_t start, uint32_t count, R dt)
{
#pragma omp parallel for schedule(static)
    for (long long k = 0; k < (long long)count; ++k) {
        long long i = (long long)start + k;
        R* P = pos + 4 * i;
        R* V = vel + 4 * i;
        R p[3], v[3], dr[3];
        for (int a = 0; a < 3; ++a) {
            p[a] = P[a];
            v[a] = V[a];
        }
        for (int a = 0; a < 3; ++a) dr[a] = dt * v[a];
        for (int a = 0; a < 3; ++a) p[a] += dr[a];
        RS(apply_boundaries)(cfg, p, v, dr, (R)0);
        for (int a = 0; a < 3; ++a) {
            P[a] = p[a];
            V[a] = v[a];
        }
    }
}

/* reverseFilamentsKernel (simulation/particles_kernel_impl.cuh:820-857):
 * a filament is reversed when its uniform is <= the probability. */
void RS(nwo_reverse)(const NwConfig* cfg, R* force, R* force_old, R* vel, R* pos, const float* uniform,
                     uint32_t num_filaments)
{
    const uint32_t L = cfg->filament_size;
    for (uint32_t w = 0; w < num_filaments; ++w) {
        if (uniform[w] > cfg->reverse_probability) continue;
        for (uint32_t q = 0; q < L / 2; ++q) {
            size_t i = (size_t)w * L + q, j = (size_t)w * L + L - 1 - q;
            R* arrs[4] = {pos, vel, force, force_old};
            for (int k = 0; k < 4; ++k)
                for (int c = 0; c < 4; ++c) {
                    R t = arrs[k][4 * i + c];
                    arrs[k][4 * i + c] = arrs[k][4 * j + c];
                    arrs[k][4 * j + c] = t;
                }
        }
    }
}

/* langevinKernel (simulation/particles_kernel_impl.cuh:859-874). */
void RS(nwo_langevin)(const NwConfig* cfg, R* force, const R* vel, const R* noise, uint32_t n)
{
    const R gamma = (R)cfg->gamma;
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < (long long)n; ++i) {
        for (int a = 0; a < 3; ++a) {
            R f = (R)0 - gamma * vel[4 * i + a];
            f += noise[4 * i + a];
            force[4 * i + a] += f;
        }
        if (nwo_fscale) {
            const R* v = vel + 4 * i;
            const R* z = noise + 4 * i;
            nwo_fscale[i] += fabs((double)gamma) * sqrt((double)v[0] * v[0] + (double)v[1] * v[1] + (double)v[2] * v[2])
                           + sqrt((double)z[0] * z[0] + (double)z[1] * z[1] + (double)z[2] * z[2]);
        }
    }
}

/* getTangent (simulation/particles_kernel_impl.cuh:303-309). */
static void RS(tangent)(const NwConfig* cfg, const R* a, const R* b, R* out)
{
    R rel[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
    R d = RS(length_periodic)(cfg, rel);
    out[0] = rel[0] / d;
    out[1] = rel[1] / d;
    out[2] = rel[2] / d;
    out[3] = 0;
}

/* Archived harmonic bond (NWWormsKernel_InternalForce.h:37-59) of bead i to
 * bead j: dr = r_j - r_i (minimum image), F_i -= (-(k (|dr| - r0)) / |dr|) dr. */
static void RS(wca_bond)(const NwConfig* cfg, const R* ri, const R* rj, R f[3], size_t i)
{
    R dr[3] = {rj[0] - ri[0], rj[1] - ri[1], rj[2] - ri[2]};
    RS(length_periodic)(cfg, dr);
    R r = RS(rsqrt_len)(RS(dot3)(dr, dr));
    R fm = -((R)cfg->bond_k * (r - (R)cfg->bond_r0)) / r;
    for (int a = 0; a < 3; ++a) f[a] -= fm * dr[a];
    if (nwo_fscale) nwo_fscale[i] += fabs((double)cfg->bond_k) * ((double)r + fabs((double)cfg->bond_r0));
}

/* Archived tangent drive (NWWormsKernel_DriveForce.h:21-34): F_i += F_act * unit(r_{i+1} - r_i). */
static void RS(wca_drive)(const NwConfig* cfg, const R* ri, const R* rn, R f[3], size_t i)
{
    R dr[3] = {rn[0] - ri[0], rn[1] - ri[1], rn[2] - ri[2]};
    RS(length_periodic)(cfg, dr);
    R m = RS(rsqrt_len)(RS(dot3)(dr, dr));
    for (int a = 0; a < 3; ++a) f[a] += (R)cfg->activity * (dr[a] / m);
    if (nwo_fscale) nwo_fscale[i] += fabs((double)cfg->activity);
}

/* filamentKernel (simulation/particles_kernel_impl.cuh:751-818): bending
 * U = k (1 - cos theta) over consecutive bond pairs, forces accumulated in
 * triple order p = 0 .. size-3; tangents head / central / tail (the tail
 * tangent is skipped when size == 3, as in the reference's else-if).
 * WCA_WORMS then adds bonds to +1 and -1 and the tangent drive per bead. */
void RS(nwo_filament)(const NwConfig* cfg, R* force, R* tangent, const R* pos, uint32_t num_filaments)
{
    const uint32_t L = cfg->filament_size;
    const R kb = (R)cfg->bend_k;
#pragma omp parallel for schedule(static)
    for (long long w = 0; w < (long long)num_filaments; ++w) {
        const size_t head = (size_t)w * L;
        for (uint32_t p = 0; L >= 3 && p < L - 2; ++p) {
            size_t i = head + p;
            const R* ri = pos + 4 * i;
            const R* rj = pos + 4 * (i + 1);
            const R* rk = pos + 4 * (i + 2);
            R rij[3], rjk[3];
            for (int a = 0; a < 3; ++a) {
                rij[a] = rj[a] - ri[a];
                rjk[a] = rk[a] - rj[a];
            }
            R dij = RS(length_periodic)(cfg, rij);
            R djk = RS(length_periodic)(cfg, rjk);
            R dd = RS(dot3)(rij, rjk);
            R A = kb / (dij * djk);
            R rr_ij = RS(dot3)(rij, rij), rr_jk = RS(dot3)(rjk, rjk);
            R fi[3], fj[3], fk[3];
            for (int a = 0; a < 3; ++a) {
                R B = (rij[a] * dd) / rr_ij;
                R C = (rjk[a] * dd) / rr_jk;
                fi[a] = -A * (rjk[a] - B);
                fk[a] = -A * (C - rij[a]);
                fj[a] = -fi[a] - fk[a];
            }
            for (int a = 0; a < 3; ++a) {
                force[4 * i + a] += fi[a];
                force[4 * (i + 1) + a] += fj[a];
                force[4 * (i + 2) + a] += fk[a];
            }
            if (nwo_fscale) {
                /* per component A (|r_jk| + |r_ij| |r_jk| / |r_ij|) for F_i and
                 * A (|r_ij| + |r_jk| |r_ij| / |r_jk|) for F_k: the magnitudes
                 * of the projections before they cancel */
                double Ad = fabs((double)A), si = 0, sk = 0;
                for (int a = 0; a < 3; ++a) {
                    double ui = Ad * (fabs((double)rjk[a]) + fabs((double)rij[a]) * (double)djk / (double)dij);
                    double uk = Ad * (fabs((double)rij[a]) + fabs((double)rjk[a]) * (double)dij / (double)djk);
                    si += ui * ui;
                    sk += uk * uk;
                }
                nwo_fscale[i] += sqrt(si);
                nwo_fscale[i + 2] += sqrt(sk);
                nwo_fscale[i + 1] += sqrt(si) + sqrt(sk);
            }
            force[4 * i + 3] += 0;
            RS(tangent)(cfg, ri, rk, tangent + 4 * (i + 1));
            if (p == 0) RS(tangent)(cfg, ri, rj, tangent + 4 * i);
            else if (p == L - 3) RS(tangent)(cfg, rj, rk, tangent + 4 * (i + 2));
        }
        if (cfg->model == NW_MODEL_WCA_WORMS) {
            for (uint32_t c = 0; c < L; ++c) {
                size_t i = head + c;
                R f[3] = {force[4 * i], force[4 * i + 1], force[4 * i + 2]};
                if (c + 1 < L) RS(wca_bond)(cfg, pos + 4 * i, pos + 4 * (i + 1), f, i);
                if (c > 0) RS(wca_bond)(cfg, pos + 4 * i, pos + 4 * (i - 1), f, i);
                if (c + 1 < L) RS(wca_drive)(cfg, pos + 4 * i, pos + 4 * (i + 1), f, i);
                for (int a = 0; a < 3; ++a) force[4 * i + a] = f[a];
            }
        }
    }
}

/* ---- pair forces ------------------------------------------------------------ */

/* bondHookean (simulation/particles_kernel_impl.cuh:466-473). */
static void RS(ref_bond)(const NwConfig* cfg, const R* ra, const R* rb, R out[3])
{
    R rel[3] = {rb[0] - ra[0], rb[1] - ra[1], rb[2] - ra[2]};
    R d = RS(length_periodic)(cfg, rel);
    R s = -(R)cfg->bond_k * ((R)cfg->bond_r0 - d);
    for (int a = 0; a < 3; ++a) out[a] = s * (rel[a] / d);
}

/* collideParticles (simulation/particles_kernel_impl.cuh:427-462). */
static void RS(ref_collide)(const NwConfig* cfg, const R* ra, const R* rb, const R* va, const R* vb, R out[3])
{
    R rel[3] = {rb[0] - ra[0], rb[1] - ra[1], rb[2] - ra[2]};
    R d = RS(length_periodic)(cfg, rel);
    R cd = (R)cfg->radius + (R)cfg->radius;
    out[0] = out[1] = out[2] = 0;
    if (d < cd) {
        R nrm[3] = {rel[0] / d, rel[1] / d, rel[2] / d};
        R rv[3] = {vb[0] - va[0], vb[1] - va[1], vb[2] - va[2]};
        R vn = RS(dot3)(rv, nrm);
        R sp = -(R)cfg->spring * (cd - d);
        for (int a = 0; a < 3; ++a) {
            R tv = rv[a] - vn * nrm[a];
            out[a] = sp * nrm[a];
            out[a] += (R)cfg->damping * rv[a];
            out[a] += (R)cfg->shear * tv;
        }
    }
}

/* extensileForce (simulation/particles_kernel_impl.cuh:477-487). */
static void RS(ref_extensile)(const NwConfig* cfg, const R* ra, const R* rb, const R* ta, const R* tb, R out[3])
{
    R rel[3] = {rb[0] - ra[0], rb[1] - ra[1], rb[2] - ra[2]};
    R d = RS(length_periodic)(cfg, rel);
    out[0] = out[1] = out[2] = 0;
    if (RS(dot3)(ta, tb) < (R)-0.5) {
        R den = (R)2 * d;
        for (int a = 0; a < 3; ++a) out[a] = (-(R)cfg->activity * (ta[a] - tb[a])) / den;
    }
}

/* Force scale of one REF_DEM neighbour (bond or contact, plus the
 * extensile term between filaments): the term magnitudes before their
 * differences cancel. */
static double RS(ref_term_scale)(const NwConfig* cfg, const R* ra, const R* rb, const R* va, const R* vb, const R* ta,
                                 const R* tb, int same, int bonded)
{
    R rel[3] = {rb[0] - ra[0], rb[1] - ra[1], rb[2] - ra[2]};
    double d = (double)RS(length_periodic)(cfg, rel), out = 0;
    if (bonded) {
        out = fabs((double)cfg->bond_k) * (fabs((double)cfg->bond_r0) + d);
    } else {
        double cd = 2.0 * (double)cfg->radius;
        if (d < cd) {
            double sv = sqrt((double)va[0] * va[0] + (double)va[1] * va[1] + (double)va[2] * va[2])
                      + sqrt((double)vb[0] * vb[0] + (double)vb[1] * vb[1] + (double)vb[2] * vb[2]);
            out = fabs((double)cfg->spring) * (cd + d) + fabs((double)cfg->damping) * sv + 2.0 * fabs((double)cfg->shear) * sv;
        }
    }
    if (!same && RS(dot3)(ta, tb) < (R)-0.5) {
        double st = sqrt((double)ta[0] * ta[0] + (double)ta[1] * ta[1] + (double)ta[2] * ta[2])
                  + sqrt((double)tb[0] * tb[0] + (double)tb[1] * tb[1] + (double)tb[2] * tb[2]);
        out += fabs((double)cfg->activity) * st / (2.0 * d);
    }
    return out;
}

/* Grid coordinate of a position (calcGridPos, :231-238), FP32 arithmetic. */
static void RS(grid_pos)(const NwConfig* cfg, const R* p, int g[3])
{
    for (int a = 0; a < 3; ++a) {
        float d = (float)p[a] - cfg->origin[a];
        float q = d / cfg->cell_size[a];
        float fl = floorf(q);
        g[a] = (fl != fl) ? 0 : (fl >= 2147483648.0f ? 2147483647 : (fl < -2147483648.0f ? (-2147483647 - 1) : (int)fl));
    }
}

static uint32_t RS(mask_hash)(const NwConfig* cfg, int gx, int gy, int gz)
{
    uint32_t x = (uint32_t)gx & (cfg->grid[0] - 1u);
    uint32_t y = (uint32_t)gy & (cfg->grid[1] - 1u);
    uint32_t z = (uint32_t)gz & (cfg->grid[2] - 1u);
    uint32_t zy = (uint32_t)((uint64_t)(z & 0xffffffu) * (uint64_t)(cfg->grid[1] & 0xffffffu));
    return (uint32_t)((uint64_t)(zy & 0xffffffu) * (uint64_t)(cfg->grid[0] & 0xffffffu)) +
           (uint32_t)((uint64_t)(y & 0xffffffu) * (uint64_t)(cfg->grid[0] & 0xffffffu)) + x;
}

/* REF_DEM: collideFilamentsKernel + collideCell (:694-744, 492-556).  All 27
 * offsets are visited in z, y, x order; a cell reached by several offsets
 * (grid extent below 3 under the power-of-two mask) is summed once per offset. */
static void RS(pair_ref)(const NwConfig* cfg, R* force, const R* sp, const R* sv, const R* st,
                         const uint32_t* sorted_index, const uint32_t* cell_start, const uint32_t* cell_end,
                         uint32_t n)
{
    const uint32_t L = cfg->filament_size;
#pragma omp parallel for schedule(dynamic, 256)
    for (long long p = 0; p < (long long)n; ++p) {
        const R* r = sp + 4 * p;
        const R* v = sv + 4 * p;
        const R* t = st + 4 * p;
        int g[3];
        RS(grid_pos)(cfg, r, g);
        const uint32_t fI = sorted_index[p] / L, cI = sorted_index[p] % L;
        R total[3] = {0, 0, 0};
        for (int z = -1; z <= 1; ++z)
            for (int y = -1; y <= 1; ++y)
                for (int x = -1; x <= 1; ++x) {
                    uint32_t h = RS(mask_hash)(cfg, g[0] + x, g[1] + y, g[2] + z);
                    R cs[3] = {0, 0, 0};
                    uint32_t s0 = cell_start[h];
                    if (s0 != NWO_EMPTY) {
                        uint32_t s1 = cell_end[h];
                        for (uint32_t j = s0; j < s1; ++j) {
                            if (j == (uint32_t)p) continue;
                            const R* r2 = sp + 4 * (size_t)j;
                            const R* v2 = sv + 4 * (size_t)j;
                            const R* t2 = st + 4 * (size_t)j;
                            uint32_t fJ = sorted_index[j] / L, cJ = sorted_index[j] % L;
                            int same = fI == fJ;
                            R f[3];
                            if (same && ((cI + 1u == cJ) || (cI - 1u == cJ))) RS(ref_bond)(cfg, r, r2, f);
                            else RS(ref_collide)(cfg, r, r2, v, v2, f);
                            for (int a = 0; a < 3; ++a) cs[a] += f[a];
                            if (nwo_fscale)
                                nwo_fscale[sorted_index[p]] +=
                                    RS(ref_term_scale)(cfg, r, r2, v, v2, t, t2, same, same && ((cI + 1u == cJ) || (cI - 1u == cJ)));
                            if (!same) {
                                RS(ref_extensile)(cfg, r, r2, t, t2, f);
                                for (int a = 0; a < 3; ++a) cs[a] += f[a];
                            }
                        }
                    }
                    for (int a = 0; a < 3; ++a) total[a] += cs[a];
                }
        size_t o = sorted_index[p];
        for (int a = 0; a < 3; ++a) force[4 * o + a] += total[a];
    }
}

/* Archived WCA / LJ pair magnitude (NWDeviceFunctions.h:73-76) with the
 * parameter derivation of NWWormsParameters.h:135-156:
 * f(rr) = 24 eps sigma^6 (2 sigma^6 / rr^7 - 1 / rr^4); F_i += f (r_i - r_j). */
static R RS(lj_mag)(const NwConfig* cfg, R rr)
{
    R s6 = (R)pow((double)cfg->lj_sigma, 6.0);
    R amp = (R)24 * (R)cfg->lj_epsilon * s6;
    R two_s6 = (R)2 * s6;
    R rr4 = rr * rr * rr * rr;
    R rr7 = rr * rr * rr * rr * rr * rr * rr;
    return amp * ((two_s6 / rr7) - ((R)1 / rr4));
}

static int RS(wca_excluded)(const NwConfig* cfg, uint32_t a, uint32_t b)
{
    const uint32_t L = cfg->filament_size;
    if (a / L != b / L) return 0;
    int d = (int)(a % L) - (int)(b % L);
    if (d < 0) d = -d;
    return d <= cfg->lj_exclude;
}

static int RS(axis_cells)(const NwConfig* cfg, int a, int g, int out[3])
{
    /* distinct neighbour cells along one axis (modulo wrap / clamp) */
    const int G = (int)cfg->grid[a];
    int cnt = 0;
    for (int o = -1; o <= 1; ++o) {
        int c = g + o;
        if (cfg->boundary[a] == NW_PERIODIC) {
            c %= G;
            if (c < 0) c += G;
        } else if (c < 0 || c >= G) {
            continue;
        }
        int dup = 0;
        for (int k = 0; k < cnt; ++k) dup |= out[k] == c;
        if (!dup) out[cnt++] = c;
    }
    return cnt;
}

/* WCA_WORMS pair pass: every distinct neighbour cell once, same-filament
 * pairs with |i - j| <= lj_exclude skipped (NWWormsKernel_InternalForce.h:196-208),
 * repulsive cut at lj_rcut (NWWormsKernel_LennardJones.h:38-50). */
static void RS(pair_wca)(const NwConfig* cfg, R* force, const R* sp, const uint32_t* sorted_index,
                         const uint32_t* cell_start, const uint32_t* cell_end, uint32_t n)
{
    const R rc2 = (R)cfg->lj_rcut * (R)cfg->lj_rcut;
#pragma omp parallel for schedule(dynamic, 256)
    for (long long p = 0; p < (long long)n; ++p) {
        const R* r = sp + 4 * p;
        int g[3], cx[3], cy[3], cz[3];
        RS(grid_pos)(cfg, r, g);
        /* the particle's own cell coordinates are those of its hash */
        for (int a = 0; a < 3; ++a) {
            int G = (int)cfg->grid[a];
            if (cfg->boundary[a] == NW_PERIODIC) {
                long long m = (long long)g[a] % G;
                if (m < 0) m += G;
                g[a] = (int)m;
            } else {
                if (g[a] < 0) g[a] = 0;
                if (g[a] >= G) g[a] = G - 1;
            }
        }
        int nx = RS(axis_cells)(cfg, 0, g[0], cx);
        int ny = RS(axis_cells)(cfg, 1, g[1], cy);
        int nz = RS(axis_cells)(cfg, 2, g[2], cz);
        const uint32_t me = sorted_index[p];
        R f[3] = {0, 0, 0};
        for (int kz = 0; kz < nz; ++kz)
            for (int ky = 0; ky < ny; ++ky)
                for (int kx = 0; kx < nx; ++kx) {
                    uint32_t h = ((uint32_t)cz[kz] * cfg->grid[1] + (uint32_t)cy[ky]) * cfg->grid[0] + (uint32_t)cx[kx];
                    uint32_t s0 = cell_start[h];
                    if (s0 == NWO_EMPTY) continue;
                    uint32_t s1 = cell_end[h];
                    for (uint32_t j = s0; j < s1; ++j) {
                        if (j == (uint32_t)p) continue;
                        if (RS(wca_excluded)(cfg, me, sorted_index[j])) continue;
                        const R* r2 = sp + 4 * (size_t)j;
                        R dr[3] = {r2[0] - r[0], r2[1] - r[1], r2[2] - r[2]};
                        RS(length_periodic)(cfg, dr);
                        R rr = RS(dot3)(dr, dr);
                        if (rr > rc2) continue;
                        R fm = RS(lj_mag)(cfg, rr);
                        for (int a = 0; a < 3; ++a) f[a] -= fm * dr[a];
                        if (nwo_fscale) {
                            double rrd = (double)rr, s6 = pow((double)cfg->lj_sigma, 6.0);
                            double amp = fabs(24.0 * (double)cfg->lj_epsilon * s6);
                            nwo_fscale[me] += amp * (2.0 * s6 / pow(rrd, 7.0) + 1.0 / (rrd * rrd * rrd * rrd)) * sqrt(rrd);
                        }
                    }
                }
        for (int a = 0; a < 3; ++a) force[4 * (size_t)me + a] += f[a];
    }
}

void RS(nwo_pair)(const NwConfig* cfg, R* force, const R* pos, const R* vel, const R* tangent,
                  const uint32_t* sorted_index, const uint32_t* cell_start, const uint32_t* cell_end, uint32_t n)
{
    /* reorderDataAndFindCellStartD's gather (:406-420) */
    R* sp = (R*)malloc(sizeof(R) * 4 * (size_t)n);
    R* sv = NULL;
    R* st = NULL;
    int ref = cfg->model == NW_MODEL_REF_DEM;
    if (ref) {
        sv = (R*)malloc(sizeof(R) * 4 * (size_t)n);
        st = (R*)malloc(sizeof(R) * 4 * (size_t)n);
    }
    for (uint32_t p = 0; p < n; ++p) {
        size_t o = sorted_index[p];
        for (int c = 0; c < 4; ++c) {
            sp[4 * (size_t)p + c] = pos[4 * o + c];
            if (ref) {
                sv[4 * (size_t)p + c] = vel[4 * o + c];
                st[4 * (size_t)p + c] = tangent[4 * o + c];
            }
        }
    }
    if (ref) RS(pair_ref)(cfg, force, sp, sv, st, sorted_index, cell_start, cell_end, n);
    else RS(pair_wca)(cfg, force, sp, sorted_index, cell_start, cell_end, n);
    free(sp);
    free(sv);
    free(st);
}

void RS(nwo_pair_wca_bruteforce)(const NwConfig* cfg, R* force, const R* pos, uint32_t n)
{
    const R rc2 = (R)cfg->lj_rcut * (R)cfg->lj_rcut;
    for (uint32_t i = 0; i < n; ++i) {
        R f[3] = {0, 0, 0};
        for (uint32_t j = 0; j < n; ++j) {
            if (j == i || RS(wca_excluded)(cfg, i, j)) continue;
            R dr[3] = {pos[4 * j] - pos[4 * i], pos[4 * j + 1] - pos[4 * i + 1], pos[4 * j + 2] - pos[4 * i + 2]};
            RS(length_periodic)(cfg, dr);
            R rr = RS(dot3)(dr, dr);
            if (rr > rc2) continue;
            R fm = RS(lj_mag)(cfg, rr);
            for (int a = 0; a < 3; ++a) f[a] -= fm * dr[a];
        }
        for (int a = 0; a < 3; ++a) force[4 * i + a] += f[a];
    }
}

/* ---- SRD -------------------------------------------------------------------- */

void RS(nwo_srd_shift)(const NwConfig* cfg, uint64_t step, float shift[3])
{
    float u[4];
    nwo_uniform4(cfg->seed, 0u, step, NWO_RNG_SRD_SHIFT, u);
    for (int a = 0; a < 3; ++a) shift[a] = (cfg->srd_shift_lo + u[a]) * cfg->srd_cell_size[a];
    if (cfg->dim < 3) shift[2] = 0.0f;
}

/* _solventUpdate (simulation/particleSystem.cpp:341-413) with the cell
 * kernels isokineticThermostatSRD (:605-637), cellCenterOfMomentumSRD
 * (:560-594), collideSolventKernel + rotate2D (:640-691) and
 * solvent_integrator (:145-205).  Members of a cell are visited in stable
 * (hash, index) order, as after thrust::sort_by_key. */
void RS(nwo_srd)(const NwConfig* cfg, R* pos, R* vel, uint32_t n_beads, uint32_t n_solvent, const float shift[3],
                 const float* rot_uniform, uint64_t step, R dt_srd, uint32_t* sorted_index_out,
                 uint32_t* cell_start_out, uint32_t* cell_end_out, R* cell_mean_out)
{
    const uint32_t n = n_beads + n_solvent;
    const uint32_t C = nwo_num_srd_cells(cfg);
    uint32_t* hash = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)(n ? n : 1));
    uint32_t* idx = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)(n ? n : 1));
    uint32_t* cs = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)C);
    uint32_t* ce = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)C);
    float* fp = (float*)malloc(sizeof(float) * 4 * (size_t)(n ? n : 1));
    for (size_t k = 0; k < 4 * (size_t)n; ++k) fp[k] = (float)pos[k];
    nwo_calc_hash_srd(cfg, fp, n, shift, hash, idx);
    nwo_sort_by_key(hash, idx, n);
    for (uint32_t c = 0; c < C; ++c) ce[c] = NWO_EMPTY;
    nwo_cell_bounds(hash, n, C, cs, ce);
    const int ref = cfg->srd_thermostat == NW_SRD_THERMO_REF_LAB;
    const R kT = (R)cfg->srd_kT;
#pragma omp parallel for schedule(dynamic, 1024)
    for (long long c = 0; c < (long long)C; ++c) {
        R u[3] = {0, 0, 0};
        uint32_t s0 = cs[c];
        if (s0 != NWO_EMPTY) {
            uint32_t s1 = ce[c];
            if (ref) {
                R E = 0;
                for (uint32_t k = s0; k < s1; ++k) {
                    const R* V = vel + 4 * (size_t)idx[k];
                    E += ((R)0.5 * V[3]) * (V[0] * V[0] + V[1] * V[1] + V[2] * V[2]);
                }
                R lam = (R)sqrt((double)(kT / E));
                for (uint32_t k = s0; k < s1; ++k) {
                    R* V = vel + 4 * (size_t)idx[k];
                    for (int a = 0; a < 3; ++a) V[a] = lam * V[a];
                }
            }
            R M = 0;
            for (uint32_t k = s0; k < s1; ++k) {
                const R* V = vel + 4 * (size_t)idx[k];
                R m = V[3];
                for (int a = 0; a < 3; ++a) u[a] += m * V[a];
                M += m;
            }
            if (M > 0) {
                R inv = (R)1 / M;
                for (int a = 0; a < 3; ++a) u[a] *= inv;
            }
            float uu;
            if (rot_uniform) uu = rot_uniform[c];
            else {
                float u4[4];
                nwo_uniform4(cfg->seed, (uint32_t)c, step, NWO_RNG_SRD_ROT, u4);
                uu = u4[0];
            }
            int sign = 2 * (int)(uu > 0.5f) - 1;
            float ang = (float)sign * cfg->srd_alpha;
            R sa = (R)((sizeof(R) == 4) ? (double)sinf(ang) : sin((double)ang));
            R ca = (R)((sizeof(R) == 4) ? (double)cosf(ang) : cos((double)ang));
            uint32_t nrot = 0;
            R ke = 0;
            for (uint32_t k = s0; k < s1; ++k) {
                uint32_t i = idx[k];
                if (i < n_beads && !cfg->srd_rotate_beads) continue;
                R* V = vel + 4 * (size_t)i;
                R dx = V[0] - u[0], dy = V[1] - u[1], dz = V[2] - u[2];
                R rx = dx * ca - dy * sa;
                R ry = dx * sa + dy * ca;
                V[0] = u[0] + rx;
                V[1] = u[1] + ry;
                V[2] = u[2] + dz;
                ke += ((R)0.5 * V[3]) * (rx * rx + ry * ry);
                ++nrot;
            }
            if (cfg->srd_thermostat == NW_SRD_THERMO_CELL_REL && nrot >= 2 && ke > 0) {
                R target = (R)(nrot - 1) * kT;
                R lam = (R)sqrt((double)(target / ke));
                for (uint32_t k = s0; k < s1; ++k) {
                    uint32_t i = idx[k];
                    if (i < n_beads && !cfg->srd_rotate_beads) continue;
                    R* V = vel + 4 * (size_t)i;
                    V[0] = u[0] + lam * (V[0] - u[0]);
                    V[1] = u[1] + lam * (V[1] - u[1]);
                }
            }
        }
        if (cell_mean_out) {
            cell_mean_out[4 * c] = u[0];
            cell_mean_out[4 * c + 1] = u[1];
            cell_mean_out[4 * c + 2] = u[2];
            cell_mean_out[4 * c + 3] = 0;
        }
    }
    RS(nwo_integrate_solvent)(cfg, pos, vel, n_beads, n_solvent, dt_srd);
    if (sorted_index_out) memcpy(sorted_index_out, idx, sizeof(uint32_t) * n);
    if (cell_start_out) memcpy(cell_start_out, cs, sizeof(uint32_t) * C);
    if (cell_end_out) memcpy(cell_end_out, ce, sizeof(uint32_t) * C);
    free(hash);
    free(idx);
    free(cs);
    free(ce);
    free(fp);
}

/* ---- the full step ------------------------------------------------------------ */

void RS(nwo_step)(const NwConfig* cfg, R* pos, R* vel, R* force, R* force_old, R* tangent, uint64_t step, R dt,
                  uint32_t* hash_out, uint32_t* sorted_index_out, uint32_t* cell_start_out, uint32_t* cell_end_out)
{
    const uint32_t M = cfg->num_filaments, L = cfg->filament_size;
    const uint32_t nb = M * L;
    const uint32_t ns = cfg->srd_enabled ? cfg->num_solvent : 0;
    const uint32_t C = nwo_num_cells(cfg);

    RS(nwo_integrate)(cfg, pos, vel, force, force_old, nb, dt);

    if (cfg->reverse_probability > 0.0f) {
        float* u = (float*)malloc(sizeof(float) * (M ? M : 1));
        for (uint32_t w = 0; w < M; ++w) {
            float u4[4];
            nwo_uniform4(cfg->seed, w, step, NWO_RNG_REVERSE, u4);
            u[w] = u4[0];
        }
        RS(nwo_reverse)(cfg, force, force_old, vel, pos, u, M);
        free(u);
    }

    if (!cfg->srd_enabled || cfg->langevin_with_srd) {
        R sigma;
        if (sizeof(R) == 4) {
            float s2 = 2.0f * cfg->gamma * cfg->kT;
            if (cfg->noise_dt_scaling) s2 = s2 / (float)dt;
            sigma = (R)sqrtf(s2);
        } else {
            double s2 = 2.0 * (double)cfg->gamma * (double)cfg->kT;
            if (cfg->noise_dt_scaling) s2 = s2 / (double)dt;
            sigma = (R)sqrt(s2);
        }
        R* noise = (R*)malloc(sizeof(R) * 4 * (size_t)(nb ? nb : 1));
#pragma omp parallel for schedule(static)
        for (long long i = 0; i < (long long)nb; ++i) {
            double z[4];
            nwo_normal4(cfg->seed, (uint32_t)i, step, NWO_RNG_LANGEVIN, z);
            noise[4 * i] = sigma * (R)z[0];
            noise[4 * i + 1] = sigma * (R)z[1];
            noise[4 * i + 2] = cfg->dim >= 3 ? sigma * (R)z[2] : (R)0;
            noise[4 * i + 3] = 0;
        }
        RS(nwo_langevin)(cfg, force, vel, noise, nb);
        free(noise);
    }

    RS(nwo_filament)(cfg, force, tangent, pos, M);

    uint32_t* hash = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)(nb ? nb : 1));
    uint32_t* idx = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)(nb ? nb : 1));
    uint32_t* cs = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)C);
    uint32_t* ce = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)C);
    float* fp = (float*)malloc(sizeof(float) * 4 * (size_t)(nb ? nb : 1));
    for (size_t k = 0; k < 4 * (size_t)nb; ++k) fp[k] = (float)pos[k];
    nwo_calc_hash(cfg, fp, nb, hash, idx);
    if (hash_out) memcpy(hash_out, hash, sizeof(uint32_t) * nb);
    nwo_sort_by_key(hash, idx, nb);
    for (uint32_t c = 0; c < C; ++c) ce[c] = NWO_EMPTY;
    nwo_cell_bounds(hash, nb, C, cs, ce);
    RS(nwo_pair)(cfg, force, pos, vel, tangent, idx, cs, ce, nb);
    if (sorted_index_out) memcpy(sorted_index_out, idx, sizeof(uint32_t) * nb);
    if (cell_start_out) memcpy(cell_start_out, cs, sizeof(uint32_t) * C);
    if (cell_end_out) memcpy(cell_end_out, ce, sizeof(uint32_t) * C);
    free(hash);
    free(idx);
    free(cs);
    free(ce);
    free(fp);

    if (cfg->srd_enabled && cfg->srd_gap > 0 && (step % cfg->srd_gap) == 0) {
        float shift[3];
        RS(nwo_srd_shift)(cfg, step, shift);
        uint32_t* order = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)(nb + ns ? nb + ns : 1));
        RS(nwo_srd)(cfg, pos, vel, nb, ns, shift, NULL, step, dt * (R)cfg->srd_gap, order, NULL, NULL, NULL);
        RS(nwo_reorder_solvent)(pos, vel, nb, ns, order);
        free(order);
    }
}

/* The engine stores the solvent in the cell order of the last collision:
 * solvent particle k after a collision is the k-th solvent entry of the
 * collision's stable (cell, index) order.  Solvent particles are identical,
 * so this relabelling changes no physics. */
void RS(nwo_reorder_solvent)(R* pos, R* vel, uint32_t n_beads, uint32_t n_solvent, const uint32_t* sorted_index)
{
    R* np_ = (R*)malloc(sizeof(R) * 4 * (size_t)(n_solvent ? n_solvent : 1));
    R* nv_ = (R*)malloc(sizeof(R) * 4 * (size_t)(n_solvent ? n_solvent : 1));
    size_t k = 0;
    for (size_t q = 0; q < (size_t)n_beads + n_solvent; ++q) {
        const uint32_t id = sorted_index[q];
        if (id < n_beads) continue;
        for (int c = 0; c < 4; ++c) {
            np_[4 * k + c] = pos[4 * (size_t)id + c];
            nv_[4 * k + c] = vel[4 * (size_t)id + c];
        }
        ++k;
    }
    memcpy(pos + 4 * (size_t)n_beads, np_, sizeof(R) * 4 * (size_t)n_solvent);
    memcpy(vel + 4 * (size_t)n_beads, nv_, sizeof(R) * 4 * (size_t)n_solvent);
    free(np_);
    free(nv_);
}
