/* CPU oracle for the periodic REPEAT fit — TEST INFRASTRUCTURE ONLY (see oracle.h).
 *
 * Each function restates the reference algorithm and cites the lines it
 * follows.  Build: gcc -O2 -ffp-contract=off -fPIC -shared (oracle/Makefile).
 */
#include "oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

static const double PI = 3.14159265358979323846;

/* VDW_RADII[Z-1] in Bohr; the reference table (repeat.py:563-578). */
static const double VDW[] = {
    2.72687, 2.23177, 2.31586, 2.59365, 3.85788, 3.63867, 3.45820, 3.30702,
    3.17852, 3.06419, 2.81853, 2.85443, 4.25094, 4.05819, 3.91835, 3.81252,
    3.72937, 3.65473, 3.60182, 3.21159, 3.11332, 2.99994, 2.97065, 2.85632,
    2.79774, 2.75144, 2.71365, 2.67774, 3.30230, 2.61066, 4.14133, 4.04401,
    3.99677, 3.97315, 3.95803, 3.91268, 3.88717, 3.44025, 3.16057, 2.95175,
    2.99049, 2.88372, 2.83270, 2.79963, 2.76750, 2.73916, 2.97443, 2.69097,
    4.21692, 4.14984, 4.17629, 4.22354, 4.25188, 4.16118, 4.26795, 3.49883,
    3.32781, 3.35993, 3.40718, 3.37789, 3.35143, 3.32592, 3.30041, 3.18230,
    3.26072, 3.23899, 3.22104, 3.20403, 3.18797, 3.17002, 3.43930, 2.96781,
    2.99522, 2.89978, 2.79113, 2.94797, 2.68341, 2.60215, 3.11143, 2.55585,
    4.10732, 4.06008, 4.12905, 4.44936, 4.48810, 4.50227, 4.62983, 3.47426,
    3.28623, 3.20875, 3.23521, 3.20781, 3.23521, 3.23521, 3.19458, 3.14261,
    3.15490, 3.13033, 3.11710, 3.10482, 3.09348, 3.06892, 3.05758, 3.04513,
    3.03268, 3.02023, 3.00778};
static const int NVDW = (int)(sizeof(VDW) / sizeof(VDW[0]));

static double radius_of(int z) { return (z >= 1 && z <= NVDW) ? VDW[z - 1] : 3.0; }

static void cross3(const double *a, const double *b, double *c) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}
static double dot3(const double *a, const double *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

/* ------------------------------------------------------------------ Ewald setup */

int orc_kspace(const double box[9], double cutoff, int kmax, double *kvecs, double *kcoefs, int cap) {
    /* repeat.py:1083 alpha; 1095-1099 reciprocal vectors (signed volume);
     * 1127-1143 k-set with kx >= 0, 0 < ksq < KMAX^2 and kcoef. */
    double bc[3], ca[3], ab[3];
    cross3(box + 3, box + 6, bc);
    cross3(box + 6, box, ca);
    cross3(box, box + 3, ab);
    double vol = dot3(box, bc);
    double rec[9];
    for (int d = 0; d < 3; ++d) {
        rec[d] = 2 * PI * bc[d] / vol;
        rec[3 + d] = 2 * PI * ca[d] / vol;
        rec[6 + d] = 2 * PI * ab[d] / vol;
    }
    double alpha = (PI / cutoff) * (PI / cutoff);
    double beta = 1.0 / (4.0 * alpha);
    int K = 0;
    int ksqmax = kmax * kmax;
    for (int kx = 0; kx <= kmax; ++kx)
        for (int ky = -kmax; ky <= kmax; ++ky)
            for (int kz = -kmax; kz <= kmax; ++kz) {
                int s = kx * kx + ky * ky + kz * kz;
                if (s >= ksqmax || s == 0) continue;
                if (K < cap) {
                    double kv[3];
                    for (int d = 0; d < 3; ++d) kv[d] = (kx * rec[d] + ky * rec[3 + d]) + kz * rec[6 + d];
                    double k2 = dot3(kv, kv);
                    kvecs[3 * K] = kv[0]; kvecs[3 * K + 1] = kv[1]; kvecs[3 * K + 2] = kv[2];
                    kcoefs[K] = (4.0 * PI / vol) * exp(-beta * k2) / k2;
                }
                ++K;
            }
    return K <= cap ? K : -K;
}

int orc_realspace_shifts(const double box[9], double cutoff, double *shifts, int cap) {
    /* repeat.py:1101-1104: nmax_i = floor(Rc / |a_i|) + 1; 815-822 order ix, iy, iz */
    int nmax[3];
    for (int i = 0; i < 3; ++i) nmax[i] = (int)floor(cutoff / sqrt(dot3(box + 3 * i, box + 3 * i))) + 1;
    int S = 0;
    for (int ix = -nmax[0]; ix <= nmax[0]; ++ix)
        for (int iy = -nmax[1]; iy <= nmax[1]; ++iy)
            for (int iz = -nmax[2]; iz <= nmax[2]; ++iz) {
                if (S < cap)
                    for (int d = 0; d < 3; ++d)
                        shifts[3 * S + d] = (ix * box[d] + iy * box[3 + d]) + iz * box[6 + d];
                ++S;
            }
    return S <= cap ? S : -S;
}

int orc_prune_shifts(const double *shifts, int S, const double *grid, int64_t M, const double *atoms,
                     int N, double cutoff, double *out, int *zero_idx) {
    /* repeat.py:1031-1069 (_prune_realspace_shifts_aabb) and 1724-1731 (zero index) */
    double gmin[3] = {1e300, 1e300, 1e300}, gmax[3] = {-1e300, -1e300, -1e300};
    double amin[3] = {1e300, 1e300, 1e300}, amax[3] = {-1e300, -1e300, -1e300};
    for (int64_t m = 0; m < M; ++m)
        for (int d = 0; d < 3; ++d) {
            double v = grid[3 * m + d];
            if (v < gmin[d]) gmin[d] = v;
            if (v > gmax[d]) gmax[d] = v;
        }
    for (int a = 0; a < N; ++a)
        for (int d = 0; d < 3; ++d) {
            double v = atoms[3 * a + d];
            if (v < amin[d]) amin[d] = v;
            if (v > amax[d]) amax[d] = v;
        }
    double R2 = cutoff * cutoff;
    int kept = 0;
    for (int s = 0; s < S; ++s) {
        double d2 = 0.0;
        for (int d = 0; d < 3; ++d) {
            double smin = amin[d] + shifts[3 * s + d], smax = amax[d] + shifts[3 * s + d];
            if (gmax[d] < smin) { double t = smin - gmax[d]; d2 += t * t; }
            else if (smax < gmin[d]) { double t = gmin[d] - smax; d2 += t * t; }
        }
        if (d2 <= R2) {
            memcpy(out + 3 * kept, shifts + 3 * s, 3 * sizeof(double));
            ++kept;
        }
    }
    if (kept == 0) { out[0] = out[1] = out[2] = 0.0; kept = 1; }
    *zero_idx = -1;
    for (int s = 0; s < kept; ++s)
        if (out[3 * s] == 0.0 && out[3 * s + 1] == 0.0 && out[3 * s + 2] == 0.0) { *zero_idx = s; break; }
    return kept;
}

/* ------------------------------------------------------------------ filter */

typedef struct {
    int nx, ny, nz;
    const double *axis;
    int A;                 /* effective atoms */
    const double *ex;      /* 3A */
    const double *rmin2, *rmin, *rmax2, *rmax;
    int near_all;          /* near proved true for every grid point */
    /* bins for the reject test */
    double bmin[3], bsize;
    int bn[3];
    const int *boff, *bidx;
    uint8_t *mask;
    int use_sqrt;
    int k0, k1;
    int64_t kept;
} filt_job;

static int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

static void *filt_work(void *p) {
    filt_job *j = (filt_job *)p;
    const double *ax = j->axis;
    int64_t kept = 0;
    for (int k = j->k0; k < j->k1; ++k)
        for (int jj = 0; jj < j->ny; ++jj)
            for (int i = 0; i < j->nx; ++i) {
                /* grid point as repeat.py:2040-2047 / 2142: (i*a0 + j*a1) + k*a2 */
                double g[3];
                for (int d = 0; d < 3; ++d) g[d] = (i * ax[d] + jj * ax[3 + d]) + k * ax[6 + d];
                int valid = 1, near = j->near_all;
                int bc[3];
                for (int d = 0; d < 3; ++d)
                    bc[d] = clampi((int)floor((g[d] - j->bmin[d]) / j->bsize), 0, j->bn[d] - 1);
                for (int dz = -1; dz <= 1 && valid; ++dz) {
                    int z2 = bc[2] + dz;
                    if (z2 < 0 || z2 >= j->bn[2]) continue;
                    for (int dy = -1; dy <= 1 && valid; ++dy) {
                        int y2 = bc[1] + dy;
                        if (y2 < 0 || y2 >= j->bn[1]) continue;
                        for (int dx = -1; dx <= 1 && valid; ++dx) {
                            int x2 = bc[0] + dx;
                            if (x2 < 0 || x2 >= j->bn[0]) continue;
                            int b = x2 + j->bn[0] * (y2 + j->bn[1] * z2);
                            for (int t = j->boff[b]; t < j->boff[b + 1]; ++t) {
                                int a = j->bidx[t];
                                double ddx = g[0] - j->ex[3 * a], ddy = g[1] - j->ex[3 * a + 1],
                                       ddz = g[2] - j->ex[3 * a + 2];
                                double d2 = (ddx * ddx + ddy * ddy) + ddz * ddz;
                                int rej = j->use_sqrt ? !(sqrt(d2) > j->rmin[a]) : (d2 <= j->rmin2[a]);
                                if (rej) { valid = 0; break; }
                            }
                        }
                    }
                }
                if (valid && !near) {
                    for (int a = 0; a < j->A; ++a) {
                        double ddx = g[0] - j->ex[3 * a], ddy = g[1] - j->ex[3 * a + 1],
                               ddz = g[2] - j->ex[3 * a + 2];
                        double d2 = (ddx * ddx + ddy * ddy) + ddz * ddz;
                        int nr = j->use_sqrt ? (sqrt(d2) <= j->rmax[a]) : (d2 <= j->rmax2[a]);
                        if (nr) { near = 1; break; }
                    }
                }
                uint8_t keep = (uint8_t)(valid && near);
                j->mask[(size_t)i + (size_t)jj * j->nx + (size_t)k * j->nx * j->ny] = keep;
                kept += keep;
            }
    j->kept = kept;
    return NULL;
}

static int64_t filter_impl(int nx, int ny, int nz, const double axis[9], int N, const double *atoms,
                           const int *Z, double vdw_factor, double vdw_max, uint8_t *mask, int threads,
                           int use_sqrt) {
    /* Effective atoms, repeat.py:1933-1969: 27 images (shift order kz, ky, kx;
     * repeat.py:787-793), atom-major, kept when inside the AABB of the corners
     * of the *grid-step* parallelepiped (axis vectors, as repeat.py:1945-1948
     * computes it) expanded by max(rmax) + 0.1. */
    double box[9];
    for (int i = 0; i < 3; ++i)
        for (int d = 0; d < 3; ++d) box[3 * i + d] = (i == 0 ? nx : (i == 1 ? ny : nz)) * axis[3 * i + d];
    double gmaxr = 5.0;
    if (N > 0) {
        gmaxr = -1e300;
        for (int a = 0; a < N; ++a) {
            double r = vdw_max * radius_of(Z[a]);
            if (r > gmaxr) gmaxr = r;
        }
    }
    double cmin[3] = {1e300, 1e300, 1e300}, cmax[3] = {-1e300, -1e300, -1e300};
    for (int c = 0; c < 8; ++c) {
        int f[3] = {(c >> 2) & 1, (c >> 1) & 1, c & 1};
        for (int d = 0; d < 3; ++d) {
            double v = (f[0] * axis[d] + f[1] * axis[3 + d]) + f[2] * axis[6 + d];
            if (v < cmin[d]) cmin[d] = v;
            if (v > cmax[d]) cmax[d] = v;
        }
    }
    double margin = gmaxr + 0.1, lmin[3], lmax[3];
    for (int d = 0; d < 3; ++d) { lmin[d] = cmin[d] - margin; lmax[d] = cmax[d] + margin; }

    double *ex = (double *)malloc(sizeof(double) * 3 * 27 * (size_t)(N > 0 ? N : 1));
    double *rmin2 = (double *)malloc(sizeof(double) * 27 * (size_t)(N > 0 ? N : 1));
    double *rmin = (double *)malloc(sizeof(double) * 27 * (size_t)(N > 0 ? N : 1));
    double *rmax2 = (double *)malloc(sizeof(double) * 27 * (size_t)(N > 0 ? N : 1));
    double *rmax = (double *)malloc(sizeof(double) * 27 * (size_t)(N > 0 ? N : 1));
    int A = 0;
    double maxrmin = 0.0;
    for (int a = 0; a < N; ++a) {
        double raw = radius_of(Z[a]);
        double rn = vdw_factor * raw, rx = vdw_max * raw;
        for (int kz = -1; kz <= 1; ++kz)
            for (int ky = -1; ky <= 1; ++ky)
                for (int kx = -1; kx <= 1; ++kx) {
                    double p[3];
                    int in = 1;
                    for (int d = 0; d < 3; ++d) {
                        double sh = (kx * box[d] + ky * box[3 + d]) + kz * box[6 + d];
                        p[d] = atoms[3 * a + d] + sh;
                        if (!(p[d] >= lmin[d] && p[d] <= lmax[d])) in = 0;
                    }
                    if (!in) continue;
                    memcpy(ex + 3 * A, p, sizeof(p));
                    rmin[A] = rn; rmin2[A] = rn * rn; rmax[A] = rx; rmax2[A] = rx * rx;
                    if (rn > maxrmin) maxrmin = rn;
                    ++A;
                }
    }
    /* near is true everywhere when one effective atom reaches every corner of the
     * grid's hull with room to spare (the hull is convex, so corners bound it) */
    int near_all = 0;
    for (int a = 0; a < A && !near_all; ++a) {
        double worst = 0.0;
        for (int c = 0; c < 8; ++c) {
            int f[3] = {(c & 1) ? nx - 1 : 0, (c & 2) ? ny - 1 : 0, (c & 4) ? nz - 1 : 0};
            double d2 = 0.0;
            for (int d = 0; d < 3; ++d) {
                double v = (f[0] * axis[d] + f[1] * axis[3 + d]) + f[2] * axis[6 + d] - ex[3 * a + d];
                d2 += v * v;
            }
            if (d2 > worst) worst = d2;
        }
        if (worst * (1.0 + 1e-9) + 1e-9 < rmax2[a]) near_all = 1;
    }
    /* reject bins: any pair in non-adjacent bins is farther apart than bsize >= max rmin */
    double bsize = (maxrmin > 0 ? maxrmin : 1.0) * (1.0 + 1e-9) + 1e-6;
    double bmin[3] = {1e300, 1e300, 1e300}, bmax[3] = {-1e300, -1e300, -1e300};
    for (int a = 0; a < A; ++a)
        for (int d = 0; d < 3; ++d) {
            if (ex[3 * a + d] < bmin[d]) bmin[d] = ex[3 * a + d];
            if (ex[3 * a + d] > bmax[d]) bmax[d] = ex[3 * a + d];
        }
    if (A == 0) for (int d = 0; d < 3; ++d) { bmin[d] = 0; bmax[d] = 0; }
    int bn[3];
    for (int d = 0; d < 3; ++d) {
        bn[d] = (int)ceil((bmax[d] - bmin[d]) / bsize) + 1;
        if (bn[d] < 1) bn[d] = 1;
        if (bn[d] > 4096) bn[d] = 4096;
    }
    /* with the bin count capped, grow the bin size so the adjacency proof still holds */
    for (int d = 0; d < 3; ++d) {
        double need = (bmax[d] - bmin[d]) / (bn[d] - 1 > 0 ? bn[d] - 1 : 1);
        if (bn[d] == 4096 && need > bsize) bsize = need * (1.0 + 1e-9);
    }
    int nb = bn[0] * bn[1] * bn[2];
    int *boff = (int *)calloc((size_t)nb + 1, sizeof(int));
    int *bidx = (int *)malloc(sizeof(int) * (size_t)(A > 0 ? A : 1));
    int *cur = (int *)malloc(sizeof(int) * (size_t)nb);
    for (int a = 0; a < A; ++a) {
        int b = 0, m = 1;
        for (int d = 0; d < 3; ++d) {
            b += m * clampi((int)floor((ex[3 * a + d] - bmin[d]) / bsize), 0, bn[d] - 1);
            m *= bn[d];
        }
        boff[b + 1]++;
    }
    for (int b = 0; b < nb; ++b) boff[b + 1] += boff[b];
    memcpy(cur, boff, sizeof(int) * (size_t)nb);
    for (int a = 0; a < A; ++a) {
        int b = 0, m = 1;
        for (int d = 0; d < 3; ++d) {
            b += m * clampi((int)floor((ex[3 * a + d] - bmin[d]) / bsize), 0, bn[d] - 1);
            m *= bn[d];
        }
        bidx[cur[b]++] = a;
    }
    if (threads < 1) threads = 1;
    if (threads > nz) threads = nz;
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)threads);
    filt_job *jobs = (filt_job *)calloc((size_t)threads, sizeof(filt_job));
    int per = (nz + threads - 1) / threads, started = 0;
    for (int t = 0; t < threads; ++t) {
        filt_job *j = &jobs[t];
        j->nx = nx; j->ny = ny; j->nz = nz; j->axis = axis; j->A = A; j->ex = ex;
        j->rmin2 = rmin2; j->rmin = rmin; j->rmax2 = rmax2; j->rmax = rmax; j->near_all = near_all;
        memcpy(j->bmin, bmin, sizeof(bmin)); j->bsize = bsize; memcpy(j->bn, bn, sizeof(bn));
        j->boff = boff; j->bidx = bidx; j->mask = mask; j->use_sqrt = use_sqrt;
        j->k0 = t * per; j->k1 = (t + 1) * per < nz ? (t + 1) * per : nz;
        if (j->k0 >= j->k1) break;
        pthread_create(&th[t], NULL, filt_work, j);
        ++started;
    }
    int64_t kept = 0;
    for (int t = 0; t < started; ++t) { pthread_join(th[t], NULL); kept += jobs[t].kept; }
    free(th); free(jobs); free(boff); free(bidx); free(cur);
    free(ex); free(rmin2); free(rmin); free(rmax2); free(rmax);
    return kept;
}

int64_t orc_filter(int nx, int ny, int nz, const double axis[9], int N, const double *atoms, const int *Z,
                   double vdw_factor, double vdw_max, uint8_t *mask, int threads) {
    /* squared-distance rule of the reference GPU filter (repeat.py:508-516) */
    return filter_impl(nx, ny, nz, axis, N, atoms, Z, vdw_factor, vdw_max, mask, threads, 0);
}

int64_t orc_filter_sqrt(int nx, int ny, int nz, const double axis[9], int N, const double *atoms,
                        const int *Z, double vdw_factor, double vdw_max, uint8_t *mask, int threads) {
    /* sqrt-distance rule of the reference CPU filter (repeat.py:2176-2177) */
    return filter_impl(nx, ny, nz, axis, N, atoms, Z, vdw_factor, vdw_max, mask, threads, 1);
}

void orc_compact(int nx, int ny, int nz, const double axis[9], const uint8_t *mask, const double *V,
                 int64_t *kept_flat, double *grid, double *Vc, int64_t M) {
    /* repeat.py:2081-2113: flat-order gather, positions (i*a0 + j*a1) + k*a2,
     * V minus its mean over kept points */
    int64_t n = (int64_t)nx * ny * nz, m = 0;
    double sum = 0.0;
    for (int64_t f = 0; f < n && m < M; ++f) {
        if (!mask[f]) continue;
        int64_t k = f / ((int64_t)nx * ny), rem = f - k * (int64_t)nx * ny;
        int64_t j = rem / nx, i = rem - j * nx;
        if (kept_flat) kept_flat[m] = f;
        for (int d = 0; d < 3; ++d)
            grid[3 * m + d] = ((double)i * axis[d] + (double)j * axis[3 + d]) + (double)k * axis[6 + d];
        Vc[m] = V[f];
        sum += V[f];
        ++m;
    }
    double mean = M > 0 ? sum / (double)M : 0.0;
    for (int64_t t = 0; t < M; ++t) Vc[t] -= mean;
}

/* ------------------------------------------------------------------ Phi */

static double phi_pair(const double *g, const double *a, int K, const double *kvecs, const double *kcoefs,
                       int S, const double *shifts, int zero_idx, double rc, double sa) {
    /* reciprocal part, repeat.py:968-981: sum_k kcoef_k cos(k . (g - a)) */
    double dx = g[0] - a[0], dy = g[1] - a[1], dz = g[2] - a[2];
    double rec = 0.0;
    for (int k = 0; k < K; ++k) {
        double kr = (dx * kvecs[3 * k] + dy * kvecs[3 * k + 1]) + dz * kvecs[3 * k + 2];
        rec += cos(kr) * kcoefs[k];
    }
    /* real-space part, repeat.py:944-966: images within Rc, r ~ 0 self image skipped */
    double real = 0.0;
    for (int s = 0; s < S; ++s) {
        double ix = a[0] + shifts[3 * s], iy = a[1] + shifts[3 * s + 1], iz = a[2] + shifts[3 * s + 2];
        double ex = g[0] - ix, ey = g[1] - iy, ez = g[2] - iz;
        double r = sqrt((ex * ex + ey * ey) + ez * ez);
        if (!(r <= rc)) continue;
        if (s == zero_idx && !(r > 1e-10)) continue;
        real += erfc(sa * r) / r;
    }
    return real + rec; /* repeat.py:998 */
}

typedef struct {
    int64_t m0, m1;
    const double *grid, *V, *atoms, *kvecs, *kcoefs, *shifts;
    int N, K, S, zero_idx;
    double rc, sa;
    double *phi_out;   /* optional: rows m0..m1 */
    double *ata, *atb, *sphi, sv;
} phi_job;

static void *phi_work(void *p) {
    phi_job *j = (phi_job *)p;
    int N = j->N;
    double *row = (double *)malloc(sizeof(double) * (size_t)N);
    for (int64_t m = j->m0; m < j->m1; ++m) {
        const double *g = j->grid + 3 * m;
        for (int a = 0; a < N; ++a)
            row[a] = phi_pair(g, j->atoms + 3 * a, j->K, j->kvecs, j->kcoefs, j->S, j->shifts, j->zero_idx,
                              j->rc, j->sa);
        if (j->phi_out) memcpy(j->phi_out + (size_t)m * N, row, sizeof(double) * (size_t)N);
        if (j->ata) {
            /* rank-1 accumulation as repeat_cpu_omp.cpp:586-604 (upper triangle; mirrored later) */
            double v = j->V[m];
            j->sv += v;
            for (int a = 0; a < N; ++a) {
                double pa = row[a];
                j->atb[a] += pa * v;
                j->sphi[a] += pa;
                double *r = j->ata + (size_t)a * N;
                for (int b = a; b < N; ++b) r[b] += pa * row[b];
            }
        }
    }
    free(row);
    return NULL;
}

void orc_phi(int64_t M, const double *grid, int N, const double *atoms, int K, const double *kvecs,
             const double *kcoefs, int S, const double *shifts, int zero_idx, double cutoff,
             double sqrt_alpha, double *phi, int threads) {
    if (threads < 1) threads = 1;
    if (threads > M) threads = (int)(M > 0 ? M : 1);
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)threads);
    phi_job *jobs = (phi_job *)calloc((size_t)threads, sizeof(phi_job));
    int64_t per = (M + threads - 1) / threads;
    int started = 0;
    for (int t = 0; t < threads; ++t) {
        phi_job *j = &jobs[t];
        j->m0 = t * per; j->m1 = (t + 1) * per < M ? (t + 1) * per : M;
        if (j->m0 >= j->m1) break;
        j->grid = grid; j->atoms = atoms; j->kvecs = kvecs; j->kcoefs = kcoefs; j->shifts = shifts;
        j->N = N; j->K = K; j->S = S; j->zero_idx = zero_idx; j->rc = cutoff; j->sa = sqrt_alpha;
        j->phi_out = phi;
        pthread_create(&th[t], NULL, phi_work, j);
        ++started;
    }
    for (int t = 0; t < started; ++t) pthread_join(th[t], NULL);
    free(th); free(jobs);
}

int orc_normal_equations(int64_t M, const double *grid, const double *V, int N, const double *atoms, int K,
                         const double *kvecs, const double *kcoefs, int S, const double *shifts, int zero_idx,
                         double cutoff, double *A, double *b, double *sum_phi, double *sum_V, int threads) {
    if (threads < 1) threads = 1;
    if (threads > M) threads = (int)(M > 0 ? M : 1);
    size_t nn = (size_t)N * N;
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)threads);
    phi_job *jobs = (phi_job *)calloc((size_t)threads, sizeof(phi_job));
    int64_t per = (M + threads - 1) / threads;
    int started = 0;
    for (int t = 0; t < threads; ++t) {
        phi_job *j = &jobs[t];
        j->m0 = t * per; j->m1 = (t + 1) * per < M ? (t + 1) * per : M;
        if (j->m0 >= j->m1) break;
        j->grid = grid; j->V = V; j->atoms = atoms; j->kvecs = kvecs; j->kcoefs = kcoefs; j->shifts = shifts;
        j->N = N; j->K = K; j->S = S; j->zero_idx = zero_idx; j->rc = cutoff;
        j->sa = sqrt((PI / cutoff) * (PI / cutoff));
        j->ata = (double *)calloc(nn, sizeof(double));
        j->atb = (double *)calloc((size_t)N, sizeof(double));
        j->sphi = (double *)calloc((size_t)N, sizeof(double));
        if (!j->ata || !j->atb || !j->sphi) return -2;
        pthread_create(&th[t], NULL, phi_work, j);
        ++started;
    }
    memset(A, 0, nn * sizeof(double));
    memset(b, 0, (size_t)N * sizeof(double));
    memset(sum_phi, 0, (size_t)N * sizeof(double));
    double sv = 0.0;
    for (int t = 0; t < started; ++t) {   /* fixed order: deterministic */
        pthread_join(th[t], NULL);
        phi_job *j = &jobs[t];
        for (size_t e = 0; e < nn; ++e) A[e] += j->ata[e];
        for (int a = 0; a < N; ++a) { b[a] += j->atb[a]; sum_phi[a] += j->sphi[a]; }
        sv += j->sv;
        free(j->ata); free(j->atb); free(j->sphi);
    }
    for (int a = 0; a < N; ++a)
        for (int c = a + 1; c < N; ++c) A[(size_t)c * N + a] = A[(size_t)a * N + c];
    /* mean correction, repeat.py:2266-2276 */
    double Mi = (double)M;
    for (int a = 0; a < N; ++a) {
        double pa = sum_phi[a] / Mi;
        for (int c = 0; c < N; ++c) A[(size_t)a * N + c] -= Mi * pa * (sum_phi[c] / Mi);
        b[a] -= Mi * pa * (sv / Mi);
    }
    *sum_V = sv;
    free(th); free(jobs);
    return 0;
}

/* ------------------------------------------------------------------ solve */

int orc_lu_solve(int n, double *A, double *b, double *x) {
    /* Gaussian elimination with partial pivoting (repeat_cpu_omp.cpp:466-495);
     * returns 1 when a pivot magnitude falls below 1e-300 (singular). */
    int sing = 0;
    for (int i = 0; i < n; ++i) {
        int p = i;
        for (int k = i + 1; k < n; ++k)
            if (fabs(A[(size_t)k * n + i]) > fabs(A[(size_t)p * n + i])) p = k;
        if (p != i) {
            for (int c = 0; c < n; ++c) {
                double t = A[(size_t)i * n + c]; A[(size_t)i * n + c] = A[(size_t)p * n + c]; A[(size_t)p * n + c] = t;
            }
            double t = b[i]; b[i] = b[p]; b[p] = t;
        }
        double piv = A[(size_t)i * n + i];
        if (fabs(piv) < 1e-300) { sing = 1; piv = piv < 0 ? -1e-300 : 1e-300; A[(size_t)i * n + i] = piv; }
        for (int k = i + 1; k < n; ++k) {
            double f = A[(size_t)k * n + i] / piv;
            if (f == 0.0) continue;
            b[k] -= f * b[i];
            for (int c = i; c < n; ++c) A[(size_t)k * n + c] -= f * A[(size_t)i * n + c];
        }
    }
    for (int i = n - 1; i >= 0; --i) {
        double s = b[i];
        for (int c = i + 1; c < n; ++c) s -= A[(size_t)i * n + c] * x[c];
        x[i] = s / A[(size_t)i * n + i];
    }
    return sing;
}

int orc_solve(int N, double *A, double *b, int n_groups, const int *group_ptr, const int *group_idx,
              const double *resp_s, const double *resp_t, double qtot, double *charges) {
    double *w = (double *)malloc(sizeof(double) * (size_t)N);
    for (int i = 0; i < N; ++i) w[i] = 1.0;
    /* symmetry folding, repeat.py:2445-2470: columns (and b, weights) of every
     * tree first, then rows, then drop linked atoms */
    for (int g = 0; g < n_groups; ++g) {
        int base = group_idx[group_ptr[g]];
        for (int t = group_ptr[g] + 1; t < group_ptr[g + 1]; ++t) {
            int l = group_idx[t];
            b[base] += b[l];
            w[base] += 1.0;
            for (int r = 0; r < N; ++r) A[(size_t)r * N + base] += A[(size_t)r * N + l];
        }
    }
    for (int g = 0; g < n_groups; ++g) {
        int base = group_idx[group_ptr[g]];
        for (int t = group_ptr[g] + 1; t < group_ptr[g + 1]; ++t) {
            int l = group_idx[t];
            for (int c = 0; c < N; ++c) A[(size_t)base * N + c] += A[(size_t)l * N + c];
        }
    }
    char *linked = (char *)calloc((size_t)N, 1);
    for (int g = 0; g < n_groups; ++g)
        for (int t = group_ptr[g] + 1; t < group_ptr[g + 1]; ++t) linked[group_idx[t]] = 1;
    int *ind = (int *)malloc(sizeof(int) * (size_t)N);
    int n = 0;
    for (int i = 0; i < N; ++i) if (!linked[i]) ind[n++] = i;
    /* bordered system with RESP on the diagonal, repeat.py:2511-2520 and 2296-2304 */
    int n1 = n + 1;
    double *As = (double *)calloc((size_t)n1 * n1, sizeof(double));
    double *bs = (double *)calloc((size_t)n1, sizeof(double));
    double *x = (double *)calloc((size_t)n1, sizeof(double));
    for (int r = 0; r < n; ++r) {
        for (int c = 0; c < n; ++c) As[(size_t)r * n1 + c] = A[(size_t)ind[r] * N + ind[c]];
        bs[r] = b[ind[r]];
        if (resp_s && resp_s[ind[r]] != 0.0) {
            As[(size_t)r * n1 + r] += resp_s[ind[r]];
            bs[r] += resp_s[ind[r]] * resp_t[ind[r]];
        }
        As[(size_t)r * n1 + n] = w[ind[r]];
        As[(size_t)n * n1 + r] = w[ind[r]];
    }
    bs[n] = qtot;
    int sing = orc_lu_solve(n1, As, bs, x);
    /* expand, repeat.py:2472-2489 */
    for (int i = 0; i < N; ++i) charges[i] = 0.0;
    for (int r = 0; r < n; ++r) charges[ind[r]] = x[r];
    for (int g = 0; g < n_groups; ++g) {
        int base = group_idx[group_ptr[g]];
        for (int t = group_ptr[g] + 1; t < group_ptr[g + 1]; ++t) charges[group_idx[t]] = charges[base];
    }
    free(w); free(linked); free(ind); free(As); free(bs); free(x);
    return sing;
}
