// Field output on the device (pybte/io_output.py:187-276): the angular
// moments of the distribution per element DOF, the element that contains
// each sampling point, and T, q_x, q_y (plus the GSIS stress trio) evaluated
// there.
#include <cuda_runtime.h>

#include "pbte_internal.cuh"

namespace {

// One thread per (DOF l, element i): m[l * nt + i] = sum_d w[d] vdf[d, i, l]
// for the three weight sets (domega, cx domega, cy domega).  Consecutive
// threads read consecutive vdf entries of one direction.
__global__ void field_moments_kernel(const double *__restrict__ vdf, int ndir, int nt, int nd,
                                     const double *__restrict__ w0, const double *__restrict__ wx,
                                     const double *__restrict__ wy, double *__restrict__ m0,
                                     double *__restrict__ mx, double *__restrict__ my) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nt * nd) return;
    const int i = t / nd, l = t % nd;
    double s0 = 0.0, sx = 0.0, sy = 0.0;
    for (int d = 0; d < ndir; ++d) {
        const double f = vdf[(size_t)d * nt * nd + t];
        s0 += w0[d] * f;
        sx += wx[d] * f;
        sy += wy[d] * f;
    }
    m0[(size_t)l * nt + i] = s0;
    mx[(size_t)l * nt + i] = sx;
    my[(size_t)l * nt + i] = sy;
}

// Bin of a coordinate: floor((v - v0) / h) clamped to [0, nb - 1], with the
// subtraction and division rounded exactly as the host rounds them when it
// fills the bins, so a point always lands in a bin its element was listed in.
__device__ __forceinline__ int bin_of(double v, double v0, double h, int nb) {
    const double c = floor(__ddiv_rn(__dsub_rn(v, v0), h));
    if (c < 0.0) return 0;
    if (c > (double)(nb - 1)) return nb - 1;
    return (int)c;
}

// One thread per sampling point (i, j) -> out[i * ny + j]: the smallest
// element index whose three sub-areas are all >= -1e-12, i.e. pybte's
// first-match-wins scan.  Only the elements listed in the point's bin are
// tested; they are listed in increasing index, and every element that can
// pass is listed there (its box, widened past the slack, covers the point),
// so the first passing candidate is the scan's answer.  Each sub-area is
// evaluated in pybte's operation order with round-to-nearest intrinsics (no
// contraction into FMA), so decisions on element edges are the reference's.
__global__ void locate_points_kernel(const double *__restrict__ tx, const double *__restrict__ ty,
                                     double x0, double y0, double hx, double hy, int nbx, int nby,
                                     const int32_t *__restrict__ bin_start, const int32_t *__restrict__ bin_items,
                                     const double *__restrict__ px, int nx, const double *__restrict__ py, int ny,
                                     int32_t *__restrict__ out) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nx * ny) return;
    const double x = px[p / ny], y = py[p % ny];
    int hit = -1;
    if (x == x && y == y) {
        const int b = bin_of(x, x0, hx, nbx) * nby + bin_of(y, y0, hy, nby);
        for (int c = bin_start[b]; c < bin_start[b + 1] && hit < 0; ++c) {
            const int k = bin_items[c];
            bool inside = true;
#pragma unroll
            for (int il = 0; il < 3; ++il) {
                const int i2 = il == 2 ? 0 : il + 1;
                const double xa = tx[3 * k + il], xb = tx[3 * k + i2];
                const double ya = ty[3 * k + il], yb = ty[3 * k + i2];
                const double t1 = __dmul_rn(x, __dsub_rn(ya, yb));
                const double t2 = __dmul_rn(y, __dsub_rn(xa, xb));
                const double t3 = __dsub_rn(__dmul_rn(xa, yb), __dmul_rn(xb, ya));
                const double area = __dmul_rn(0.5, __dadd_rn(__dsub_rn(t1, t2), t3));
                inside = inside && (area >= -1e-12);
            }
            if (inside) hit = k;
        }
    }
    out[p] = hit;
}

// One thread per sampling point: the reference coordinates of the point in
// its element (the affine map in pybte's form xi = B/A x + C/A y + D/A,
// pybte/integration.py:52-68), the Lagrange basis there from its monomial
// coefficients, and the fields as basis-weighted sums of the element's DOF
// coefficients.  Points outside the mesh get zeros.
__global__ void sample_fields_kernel(const double *__restrict__ tx, const double *__restrict__ ty,
                                     const int32_t *__restrict__ triid, const double *__restrict__ px, int nx,
                                     const double *__restrict__ py, int ny, const double *__restrict__ nodfun,
                                     const int32_t *__restrict__ mono, int nd, const double *__restrict__ m0,
                                     const double *__restrict__ mx, const double *__restrict__ my, int nt,
                                     double cv, const double *__restrict__ uq, double *__restrict__ out) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = nx * ny;
    if (p >= n) return;
    const int k = triid[p];
    double f[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    if (k >= 0) {
        const double x = px[p / ny], y = py[p % ny];
        const double x1 = tx[3 * k], x2 = tx[3 * k + 1], x3 = tx[3 * k + 2];
        const double y1 = ty[3 * k], y2 = ty[3 * k + 1], y3 = ty[3 * k + 2];
        const double A = (x2 - x1) * (y3 - y1) - (x3 - x1) * (y2 - y1);
        const double E = (x3 - x1) * (y2 - y1) - (x2 - x1) * (y3 - y1);
        const double xi = (y3 - y1) / A * x + (x1 - x3) / A * y + ((x3 - x1) * y1 - (y3 - y1) * x1) / A;
        const double eta = (y2 - y1) / E * x + (x1 - x2) / E * y + ((x2 - x1) * y1 - (y2 - y1) * x1) / E;
        for (int l = 0; l < nd; ++l) {
            double phi = 0.0;
            for (int c = 0; c < nd; ++c) {
                double m = 1.0;
                for (int a = 0; a < mono[2 * c]; ++a) m *= xi;
                for (int b = 0; b < mono[2 * c + 1]; ++b) m *= eta;
                phi += nodfun[l * nd + c] * m;
            }
            const size_t e = (size_t)l * nt + k;
            f[0] += phi * m0[e];
            f[1] += phi * mx[e];
            f[2] += phi * my[e];
            if (uq) {
                // uq rows 3..6 blocks: l_xx, l_xy, l_yx, l_yy (pybte/io_output.py:269-275)
                const double lxx = uq[(size_t)(3 * nd + l) * nt + k], lxy = uq[(size_t)(4 * nd + l) * nt + k];
                const double lyx = uq[(size_t)(5 * nd + l) * nt + k], lyy = uq[(size_t)(6 * nd + l) * nt + k];
                f[3] += phi * (-4.0 / 3.0 * lxx + 2.0 / 3.0 * lyy);
                f[4] += phi * (-lxy - lyx);
                f[5] += phi * (2.0 / 3.0 * lxx - 4.0 / 3.0 * lyy);
            }
        }
        f[0] /= cv;
    }
#pragma unroll
    for (int q = 0; q < 6; ++q) out[(size_t)q * n + p] = f[q];
}

inline int blocks_for(long long n, int th) { return (int)((n + th - 1) / th); }

}  // namespace

extern "C" int pbte_field_moments(const double *vdf, int32_t ndir, int32_t n_tris, int32_t ndof, const double *w0,
                                  const double *wx, const double *wy, double *m0, double *mx, double *my,
                                  void *stream) {
    if (!vdf || !w0 || !wx || !wy || !m0 || !mx || !my || ndir < 1 || n_tris < 1 || ndof < 1 ||
        (long long)n_tris * ndof > (1LL << 31) - 1)
        return PBTE_ERR_ARG;
    const int th = 256;
    field_moments_kernel<<<blocks_for((long long)n_tris * ndof, th), th, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
        vdf, ndir, n_tris, ndof, w0, wx, wy, m0, mx, my);
    return cudaGetLastError() == cudaSuccess ? PBTE_OK : PBTE_ERR_CUDA;
}

extern "C" int pbte_locate_points(const double *tri_x, const double *tri_y, int32_t n_tris, double x0, double y0,
                                  double hx, double hy, int32_t nbx, int32_t nby, const int32_t *bin_start,
                                  const int32_t *bin_items, const double *px, int32_t nx, const double *py,
                                  int32_t ny, int32_t *out, void *stream) {
    if (!tri_x || !tri_y || !bin_start || !bin_items || !px || !py || !out || n_tris < 1 || nx < 1 || ny < 1 ||
        nbx < 1 || nby < 1 || !(hx > 0.0) || !(hy > 0.0) || (long long)nx * ny > (1LL << 31) - 1)
        return PBTE_ERR_ARG;
    const int th = 128;
    locate_points_kernel<<<blocks_for((long long)nx * ny, th), th, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
        tri_x, tri_y, x0, y0, hx, hy, nbx, nby, bin_start, bin_items, px, nx, py, ny, out);
    return cudaGetLastError() == cudaSuccess ? PBTE_OK : PBTE_ERR_CUDA;
}

extern "C" int pbte_sample_fields(const double *tri_x, const double *tri_y, const int32_t *triid, const double *px,
                                  int32_t nx, const double *py, int32_t ny, const double *nodfun,
                                  const int32_t *mono, int32_t ndof, const double *m0, const double *mx,
                                  const double *my, int32_t n_tris, double cv, const double *uq, double *out,
                                  void *stream) {
    if (!tri_x || !tri_y || !triid || !px || !py || !nodfun || !mono || !m0 || !mx || !my || !out || nx < 1 ||
        ny < 1 || ndof < 1 || ndof > 15 || n_tris < 1 || (long long)nx * ny > (1LL << 31) - 1)
        return PBTE_ERR_ARG;
    const int th = 128;
    sample_fields_kernel<<<blocks_for((long long)nx * ny, th), th, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
        tri_x, tri_y, triid, px, nx, py, ny, nodfun, mono, ndof, m0, mx, my, n_tris, cv, uq, out);
    return cudaGetLastError() == cudaSuccess ? PBTE_OK : PBTE_ERR_CUDA;
}
