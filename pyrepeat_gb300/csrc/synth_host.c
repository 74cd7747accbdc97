/* Host helper for the synthetic-cube generator: the real-space Ewald sum of a
 * set of point charges on every point of a cube grid.
 *
 *   V(g) = sum_a q_a sum_s [|g - a - s| <= Rc] erfc(sqrt(alpha) r) / r
 *
 * with the r ~ 0 self image skipped, the rule of repeat.py:944-966.  Grid
 * point (i, j, k) is i*ax0 + j*ax1 + k*ax2 and its value lands at flat index
 * i + j*nx + k*nx*ny.  Work is split over z-layers across pthreads.
 * This is test-data generation, not part of the fit.
 */
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    int nx, ny, nz;
    const double *ax;
    int n;
    const double *img;   /* per (atom, shift) image position, 3 doubles, compacted */
    const double *imgq;  /* charge of that image */
    const int *imgself;  /* 1 if the image is the zero shift */
    int nimg;
    double rc2, sa;
    double *out;
    int k0, k1;
} job_t;

static void *work(void *p) {
    job_t *j = (job_t *)p;
    const double *ax = j->ax;
    int *cand = (int *)malloc(sizeof(int) * (size_t)(j->nimg > 0 ? j->nimg : 1));
    const double rc = sqrt(j->rc2);
    /* per grid row (fixed j, k): only images within Rc of the row's segment can
     * contribute, so each point scans that short candidate list */
    double L2 = ax[0] * ax[0] + ax[1] * ax[1] + ax[2] * ax[2];
    for (int k = j->k0; k < j->k1; ++k) {
        for (int jj = 0; jj < j->ny; ++jj) {
            double bx = ax[3] * jj + ax[6] * k, by = ax[4] * jj + ax[7] * k, bz = ax[5] * jj + ax[8] * k;
            int nc = 0;
            for (int t = 0; t < j->nimg; ++t) {
                double px = j->img[3 * t] - bx, py = j->img[3 * t + 1] - by, pz = j->img[3 * t + 2] - bz;
                double u = (px * ax[0] + py * ax[1] + pz * ax[2]) / L2;   /* position along the row */
                if (u < 0) u = 0;
                if (u > j->nx - 1) u = j->nx - 1;
                double dx = px - u * ax[0], dy = py - u * ax[1], dz = pz - u * ax[2];
                if (dx * dx + dy * dy + dz * dz <= (rc + 1e-9) * (rc + 1e-9)) cand[nc++] = t;
            }
            for (int i = 0; i < j->nx; ++i) {
                double gx = ax[0] * i + ax[3] * jj + ax[6] * k;
                double gy = ax[1] * i + ax[4] * jj + ax[7] * k;
                double gz = ax[2] * i + ax[5] * jj + ax[8] * k;
                double acc = 0.0;
                for (int c = 0; c < nc; ++c) {
                    int t = cand[c];
                    double dx = gx - j->img[3 * t];
                    double dy = gy - j->img[3 * t + 1];
                    double dz = gz - j->img[3 * t + 2];
                    double r2 = dx * dx + dy * dy + dz * dz;
                    if (r2 > j->rc2) continue;
                    double r = sqrt(r2);
                    if (j->imgself[t] && r <= 1e-10) continue;
                    acc += j->imgq[t] * erfc(j->sa * r) / r;
                }
                j->out[(size_t)i + (size_t)jj * j->nx + (size_t)k * j->nx * j->ny] = acc;
            }
        }
    }
    free(cand);
    return NULL;
}

int synth_realspace_grid(int nx, int ny, int nz, const double *axis, int n, const double *atoms,
                         const double *q, int S, const double *shifts, double rc,
                         double sqrt_alpha, int threads, double *out) {
    if (nx <= 0 || ny <= 0 || nz <= 0 || n < 0 || S <= 0) return -1;
    /* keep only images that can reach the cell: distance from the image to
     * the cell's bounding box must be <= Rc */
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int c = 0; c < 8; ++c) {
        double f0 = (c & 1) ? nx - 1 : 0, f1 = (c & 2) ? ny - 1 : 0, f2 = (c & 4) ? nz - 1 : 0;
        for (int d = 0; d < 3; ++d) {
            double v = axis[d] * f0 + axis[3 + d] * f1 + axis[6 + d] * f2;
            if (v < lo[d]) lo[d] = v;
            if (v > hi[d]) hi[d] = v;
        }
    }
    double *img = (double *)malloc(sizeof(double) * 3 * (size_t)n * S);
    double *imgq = (double *)malloc(sizeof(double) * (size_t)n * S);
    int *imgself = (int *)malloc(sizeof(int) * (size_t)n * S);
    if (!img || !imgq || !imgself) { free(img); free(imgq); free(imgself); return -2; }
    int m = 0;
    for (int a = 0; a < n; ++a) {
        for (int s = 0; s < S; ++s) {
            double p[3], d2 = 0.0;
            for (int d = 0; d < 3; ++d) {
                p[d] = atoms[3 * a + d] + shifts[3 * s + d];
                double e = 0.0;
                if (p[d] < lo[d]) e = lo[d] - p[d];
                else if (p[d] > hi[d]) e = p[d] - hi[d];
                d2 += e * e;
            }
            if (d2 > rc * rc) continue;
            img[3 * m] = p[0]; img[3 * m + 1] = p[1]; img[3 * m + 2] = p[2];
            imgq[m] = q[a];
            imgself[m] = (shifts[3 * s] == 0.0 && shifts[3 * s + 1] == 0.0 && shifts[3 * s + 2] == 0.0);
            ++m;
        }
    }
    if (threads < 1) threads = 1;
    if (threads > nz) threads = nz;
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * threads);
    job_t *jobs = (job_t *)malloc(sizeof(job_t) * threads);
    int per = (nz + threads - 1) / threads;
    int started = 0;
    for (int t = 0; t < threads; ++t) {
        jobs[t].nx = nx; jobs[t].ny = ny; jobs[t].nz = nz; jobs[t].ax = axis; jobs[t].n = n;
        jobs[t].img = img; jobs[t].imgq = imgq; jobs[t].imgself = imgself; jobs[t].nimg = m;
        jobs[t].rc2 = rc * rc; jobs[t].sa = sqrt_alpha; jobs[t].out = out;
        jobs[t].k0 = t * per; jobs[t].k1 = (t + 1) * per < nz ? (t + 1) * per : nz;
        if (jobs[t].k0 >= jobs[t].k1) break;
        pthread_create(&th[t], NULL, work, &jobs[t]);
        ++started;
    }
    for (int t = 0; t < started; ++t) pthread_join(th[t], NULL);
    free(th); free(jobs); free(img); free(imgq); free(imgself);
    return 0;
}
