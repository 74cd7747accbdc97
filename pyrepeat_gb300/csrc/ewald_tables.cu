// Ewald setup (host) and the cos/sin tables of the reciprocal-space sum.
//
// Setup follows EwaldCalculator (repeat.py:1077-1143): alpha = (pi/Rc)^2,
// reciprocal vectors b_i = 2 pi (a_j x a_k)/V with the signed volume, the k-set
// 0 <= kx <= KMAX, -KMAX <= ky, kz <= KMAX, 0 < kx^2+ky^2+kz^2 < KMAX^2 (integer
// indices, so K depends on KMAX only), kcoef = 4 pi/V exp(-k^2/4 alpha)/k^2, and
// real-space shifts |n_i| <= floor(Rc/|a_i|)+1 (repeat.py:1101-1104, 815-822).
//
// On the cube lattice a grid point is g = i a0/nx + j a1/ny + l a2/nz, so
//     k.g = 2 pi (n1 i/nx + n2 j/ny + n3 l/nz)
// exactly, and e^{i k.g} = ex[n1][i] * ey[n2][j] * ez[n3][l] with three small
// per-axis tables whose phases are reduced exactly in integers.  No per-point
// large-argument sincos is needed; atom phases k.r_a take one FP64 sincos each.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "common.cuh"
#include "df.cuh"

namespace rp {

static void cross3(const double *a, const double *b, double *c) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}

void ewald_build_host(rp_ewald *ew, const rp_grid *grid, double cutoff, int kmax, char *dst) {
    RP_REQUIRE(kmax >= 0 && kmax <= 64, "rp_ewald_setup: kmax must be in 0..64");
    RP_REQUIRE(kmax == 0 || cutoff > 0.0, "rp_ewald_setup: cutoff must be > 0");
    for (int i = 0; i < 3; ++i) RP_REQUIRE(grid->n_grid[i] > 0, "rp_ewald_setup: grid counts must be > 0");
    // kmax 0: the non-periodic basis of --fit-type 0, 1/|g - r_a| with the atom itself only
    // (repeat.py:991-994, 1263-1270): no k-vectors, the zero shift alone, alpha 0 (so the
    // real-space term erfc(0 r)/r is 1/r everywhere) and a cutoff no distance reaches
    const bool nonperiodic = kmax == 0;
    if (nonperiodic) cutoff = kNonPeriodicCutoff;
    ew->grid = *grid;
    ew->cutoff = cutoff;
    ew->kmax = kmax;
    for (int i = 0; i < 3; ++i)
        for (int d = 0; d < 3; ++d) ew->box[3 * i + d] = grid->n_grid[i] * grid->axis[3 * i + d];
    const double *a = ew->box, *b = ew->box + 3, *c = ew->box + 6;
    double bc[3], ca[3], ab[3];
    cross3(b, c, bc);
    cross3(c, a, ca);
    cross3(a, b, ab);
    double vol = a[0] * bc[0] + a[1] * bc[1] + a[2] * bc[2];
    RP_REQUIRE(std::fabs(vol) > 1e-12, "rp_ewald_setup: degenerate cell");
    ew->volume = vol;
    const double PI = 3.14159265358979323846;
    double *rec = ew->rec;
    for (int d = 0; d < 3; ++d) {
        rec[d] = 2 * PI * bc[d] / vol;
        rec[3 + d] = 2 * PI * ca[d] / vol;
        rec[6 + d] = 2 * PI * ab[d] / vol;
    }
    ew->alpha = nonperiodic ? 0.0 : (PI / cutoff) * (PI / cutoff);
    ew->sqrt_alpha = std::sqrt(ew->alpha);
    const double beta = 1.0 / (4.0 * ew->alpha);
    ew->kvec.clear();
    ew->kcoef.clear();
    ew->kidx.clear();
    const int ksqmax = kmax * kmax;
    for (int kx = 0; kx <= kmax; ++kx)
        for (int ky = -kmax; ky <= kmax; ++ky)
            for (int kz = -kmax; kz <= kmax; ++kz) {
                int s = kx * kx + ky * ky + kz * kz;
                if (s >= ksqmax || s == 0) continue;
                double kv[3];
                for (int d = 0; d < 3; ++d) kv[d] = (kx * rec[d] + ky * rec[3 + d]) + kz * rec[6 + d];
                double k2 = kv[0] * kv[0] + kv[1] * kv[1] + kv[2] * kv[2];
                ew->kvec.insert(ew->kvec.end(), kv, kv + 3);
                ew->kcoef.push_back((4.0 * PI / vol) * std::exp(-beta * k2) / k2);
                ew->kidx.push_back(kx);
                ew->kidx.push_back(ky);
                ew->kidx.push_back(kz);
            }
    ew->K = (int)ew->kcoef.size();
    int nmax[3];
    for (int i = 0; i < 3; ++i) {
        double len = std::sqrt(ew->box[3 * i] * ew->box[3 * i] + ew->box[3 * i + 1] * ew->box[3 * i + 1] +
                               ew->box[3 * i + 2] * ew->box[3 * i + 2]);
        nmax[i] = nonperiodic ? 0 : (int)std::floor(cutoff / len) + 1;
    }
    ew->shifts.clear();
    for (int ix = -nmax[0]; ix <= nmax[0]; ++ix)
        for (int iy = -nmax[1]; iy <= nmax[1]; ++iy)
            for (int iz = -nmax[2]; iz <= nmax[2]; ++iz)
                for (int d = 0; d < 3; ++d)
                    ew->shifts.push_back((ix * ew->box[d] + iy * ew->box[3 + d]) + iz * ew->box[6 + d]);
    ew->S = (int)(ew->shifts.size() / 3);

    // the device image: tables at the offsets of ewald_layout, written straight into `dst`
    // (a caller's arena) or into ew->image
    const int nx = grid->n_grid[0], ny = grid->n_grid[1], nz = grid->n_grid[2];
    int K_layout = 0;
    const size_t total = ewald_layout(grid, kmax, ew->off, &K_layout);
    RP_REQUIRE(K_layout == ew->K, "rp_ewald_setup: k-set size mismatch");
    ew->image_bytes = total;
    char *img = dst;
    if (!img) {
        ew->image.assign(total, 0);
        img = ew->image.data();
    }
    std::memcpy(img + ew->off[0], ew->kidx.data(), sizeof(int) * ew->kidx.size());
    std::memcpy(img + ew->off[1], ew->kcoef.data(), sizeof(double) * ew->kcoef.size());
    std::memcpy(img + ew->off[2], ew->kvec.data(), sizeof(double) * ew->kvec.size());
    double2 *ex = reinterpret_cast<double2 *>(img + ew->off[3]);
    double2 *ey = reinterpret_cast<double2 *>(img + ew->off[4]);
    double2 *ez = reinterpret_cast<double2 *>(img + ew->off[5]);
    // per-axis phase tables: out[i] = e^{2 pi i (n i mod L) / L}, the residue stepped exactly in
    // integers, from one table of the L roots of unity per axis
    std::vector<double2> unit;
    auto fill = [&](double2 *out, int n, int L) {
        const int step = ((n % L) + L) % L;
        int r = 0;
        for (int i = 0; i < L; ++i) {
            out[i] = unit[(size_t)r];
            r += step;
            if (r >= L) r -= L;
        }
    };
    auto roots = [&](int L) {
        unit.resize((size_t)L);
        for (int r = 0; r < L; ++r) {
            const double t = 2.0 * PI * (double)r / (double)L;
            unit[(size_t)r] = make_double2(std::cos(t), std::sin(t));
        }
    };
    roots(nx);
    for (int n = 0; n <= kmax; ++n) fill(ex + (size_t)n * nx, n, nx);
    roots(ny);
    for (int n = -kmax; n <= kmax; ++n) fill(ey + (size_t)(n + kmax) * ny, n, ny);
    roots(nz);
    for (int n = -kmax; n <= kmax; ++n) fill(ez + (size_t)(n + kmax) * nz, n, nz);
    // double-float copies over n in [-(kmax-1), kmax-1] for the separable reciprocal sum
    const int P = kmax - 1;
    float4 *exf = reinterpret_cast<float4 *>(img + ew->off[6]);
    float4 *eyf = reinterpret_cast<float4 *>(img + ew->off[7]);
    float4 *ezf = reinterpret_cast<float4 *>(img + ew->off[8]);
    for (int n = 0; n <= P; ++n)
        for (int i = 0; i < nx; ++i) {
            const double2 v = ex[(size_t)n * nx + i];
            exf[(size_t)n * nx + i] = dfa::split(v.x, v.y);
        }
    for (int n = -P; n <= P; ++n) {
        for (int j = 0; j < ny; ++j) {
            const double2 v = ey[(size_t)(n + kmax) * ny + j];
            eyf[(size_t)(n + P) * ny + j] = dfa::split(v.x, v.y);
        }
        for (int l = 0; l < nz; ++l) {
            const double2 v = ez[(size_t)(n + kmax) * nz + l];
            ezf[(size_t)(n + P) * nz + l] = dfa::split(v.x, v.y);
        }
    }
}

size_t ewald_layout(const rp_grid *grid, int kmax, size_t off[9], int *K_out) {
    int K = 0;
    const int ksqmax = kmax * kmax;
    for (int kx = 0; kx <= kmax; ++kx)
        for (int ky = -kmax; ky <= kmax; ++ky)
            for (int kz = -kmax; kz <= kmax; ++kz) {
                const int s = kx * kx + ky * ky + kz * kz;
                if (s < ksqmax && s != 0) ++K;
            }
    if (K_out) *K_out = K;
    const size_t nx = grid->n_grid[0], ny = grid->n_grid[1], nz = grid->n_grid[2];
    const size_t P1 = (size_t)kmax, nw = kmax > 0 ? 2 * (size_t)kmax - 1 : 0;  // P+1 and 2P+1, P = kmax-1
    const size_t bytes[9] = {sizeof(int) * 3 * K, sizeof(double) * K, sizeof(double) * 3 * K,
                             sizeof(double2) * (kmax + 1) * nx, sizeof(double2) * (2 * kmax + 1) * ny,
                             sizeof(double2) * (2 * kmax + 1) * nz, sizeof(float4) * P1 * nx,
                             sizeof(float4) * nw * ny, sizeof(float4) * nw * nz};
    size_t end = 0;
    for (int t = 0; t < 9; ++t) {
        off[t] = (end + 255) & ~size_t(255);
        end = off[t] + bytes[t];
    }
    return (end + 255) & ~size_t(255);
}

size_t ewald_device_bytes(const rp_ewald *ew) { return ew->image_bytes; }

void ewald_place(rp_ewald *ew, void *dev) {
    char *b = static_cast<char *>(dev);
    ew->d_kidx = reinterpret_cast<int *>(b + ew->off[0]);
    ew->d_kcoef = reinterpret_cast<double *>(b + ew->off[1]);
    ew->d_kvec = reinterpret_cast<double *>(b + ew->off[2]);
    ew->d_ex = reinterpret_cast<double2 *>(b + ew->off[3]);
    ew->d_ey = reinterpret_cast<double2 *>(b + ew->off[4]);
    ew->d_ez = reinterpret_cast<double2 *>(b + ew->off[5]);
    ew->d_exf = reinterpret_cast<float4 *>(b + ew->off[6]);
    ew->d_eyf = reinterpret_cast<float4 *>(b + ew->off[7]);
    ew->d_ezf = reinterpret_cast<float4 *>(b + ew->off[8]);
}

void ewald_build(rp_ewald *ew, const rp_grid *grid, double cutoff, int kmax) {
    ewald_build_host(ew, grid, cutoff, kmax);
    RP_CUDA(cudaMalloc(&ew->d_block, ewald_device_bytes(ew)));
    ew->owns = true;
    ewald_place(ew, ew->d_block);
    RP_CUDA(cudaMemcpy(ew->d_block, ew->image.data(), ew->image.size(), cudaMemcpyHostToDevice));
}

void ewald_free(rp_ewald *ew) {
    if (ew->owns && ew->d_block) cudaFree(ew->d_block);
    ew->d_block = nullptr;
}

void prune_shifts(const rp_ewald *ew, const double *atoms, int N, std::vector<double> &out, int &zero_idx) {
    // AABB-distance pruning as repeat.py:1031-1069, against the hull of the whole
    // grid (a superset of the kept points' box): a pruned shift has no image
    // within Rc of any grid point, so the sums are unchanged.
    const rp_grid &g = ew->grid;
    double gmin[3] = {1e300, 1e300, 1e300}, gmax[3] = {-1e300, -1e300, -1e300};
    for (int c = 0; c < 8; ++c) {
        int f0 = (c & 1) ? g.n_grid[0] - 1 : 0, f1 = (c & 2) ? g.n_grid[1] - 1 : 0, f2 = (c & 4) ? g.n_grid[2] - 1 : 0;
        for (int d = 0; d < 3; ++d) {
            double v = (f0 * g.axis[d] + f1 * g.axis[3 + d]) + f2 * g.axis[6 + d];
            gmin[d] = std::min(gmin[d], v);
            gmax[d] = std::max(gmax[d], v);
        }
    }
    double amin[3] = {1e300, 1e300, 1e300}, amax[3] = {-1e300, -1e300, -1e300};
    for (int a = 0; a < N; ++a)
        for (int d = 0; d < 3; ++d) {
            amin[d] = std::min(amin[d], atoms[3 * a + d]);
            amax[d] = std::max(amax[d], atoms[3 * a + d]);
        }
    const double R2 = ew->cutoff * ew->cutoff;
    out.clear();
    for (int s = 0; s < ew->S; ++s) {
        const double *sh = &ew->shifts[3 * (size_t)s];
        double d2 = 0.0;
        for (int d = 0; d < 3; ++d) {
            double smin = amin[d] + sh[d], smax = amax[d] + sh[d];
            if (gmax[d] < smin) d2 += (smin - gmax[d]) * (smin - gmax[d]);
            else if (smax < gmin[d]) d2 += (gmin[d] - smax) * (gmin[d] - smax);
        }
        if (d2 <= R2 * (1.0 + 1e-12)) out.insert(out.end(), sh, sh + 3);
    }
    if (out.empty()) out = {0.0, 0.0, 0.0};
    zero_idx = -1;
    for (size_t s = 0; s < out.size() / 3; ++s)
        if (out[3 * s] == 0.0 && out[3 * s + 1] == 0.0 && out[3 * s + 2] == 0.0) {
            zero_idx = (int)s;
            break;
        }
}

namespace {

__global__ void atom_tables_fp64_kernel(const double *__restrict__ kvec, const double *__restrict__ kcoef, int K,
                                        const double *__restrict__ atoms, int N, double *__restrict__ B, int ldb) {
    // B[a][k] = w_k cos(k.r_a), B[a][K+k] = w_k sin(k.r_a)
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)N * K) return;
    int a = (int)(t / K), k = (int)(t - (long long)a * K);
    double kr = (atoms[3 * a] * kvec[3 * k] + atoms[3 * a + 1] * kvec[3 * k + 1]) + atoms[3 * a + 2] * kvec[3 * k + 2];
    double s, c;
    sincos(kr, &s, &c);
    B[(size_t)a * ldb + k] = kcoef[k] * c;
    B[(size_t)a * ldb + K + k] = kcoef[k] * s;
}

__global__ void grid_tables_fp64_kernel(const int *__restrict__ kidx, int K, int kmax, const double2 *__restrict__ ex,
                                        const double2 *__restrict__ ey, const double2 *__restrict__ ez, int nx,
                                        int ny, int nz, const int32_t *__restrict__ kept, long long m0, long long rows,
                                        double *__restrict__ T, int ldt) {
    // T[m][k] = cos(k.g_m), T[m][K+k] = sin(k.g_m) from the per-axis tables
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= rows * K) return;
    long long m = t / K;
    int k = (int)(t - m * K);
    int f = kept[m0 + m];
    int layer = nx * ny;
    int l = f / layer, rem = f - l * layer, j = rem / nx, i = rem - j * nx;
    int n1 = kidx[3 * k], n2 = kidx[3 * k + 1], n3 = kidx[3 * k + 2];
    double2 a = ex[(size_t)n1 * nx + i], b = ey[(size_t)(n2 + kmax) * ny + j], c = ez[(size_t)(n3 + kmax) * nz + l];
    double re = a.x * b.x - a.y * b.y, im = a.x * b.y + a.y * b.x;
    double re2 = re * c.x - im * c.y, im2 = re * c.y + im * c.x;
    T[(size_t)m * ldt + k] = re2;
    T[(size_t)m * ldt + K + k] = im2;
}

}  // namespace

void atom_tables_fp64(const rp_ewald *ew, const double *d_atoms, int N, double *d_B, int ldb, cudaStream_t s) {
    long long n = (long long)N * ew->K;
    if (n == 0) return;
    atom_tables_fp64_kernel<<<ceil_div(n, 256), 256, 0, s>>>(ew->d_kvec, ew->d_kcoef, ew->K, d_atoms, N, d_B, ldb);
    RP_LAUNCH_CHECK();
}

void grid_tables_fp64(const rp_ewald *ew, const int32_t *d_kept, int64_t m0, int64_t rows, double *d_T, int ldt,
                      cudaStream_t s) {
    long long n = (long long)rows * ew->K;
    if (n == 0) return;
    grid_tables_fp64_kernel<<<ceil_div(n, 256), 256, 0, s>>>(ew->d_kidx, ew->K, ew->kmax, ew->d_ex, ew->d_ey, ew->d_ez,
                                                             ew->grid.n_grid[0], ew->grid.n_grid[1], ew->grid.n_grid[2],
                                                             d_kept, m0, rows, d_T, ldt);
    RP_LAUNCH_CHECK();
}

}  // namespace rp
