// Spot fits: planar background and one 2-D Gaussian per blob, a warp per blob.
//
// The reference (src/scopyon/analysis/spot_detection.py:49-141) cuts a
// (2 roi + 1)^2 region around each blob, fits a plane to its four edges by
// least squares (planar_background, :61-78), subtracts it, fits
//   g(x, y) = a1 exp(-((x - a2)^2 + (y - a3)^2) / a4)
// from a1 = 255, (a2, a3) = the intensity-weighted centre, a4 = roi / 2
// (fitgaussian, :95-103), keeps the spot when the centre lies in the region
// and returns (a2 + x0, a3 + y0, sum of g over the region, sum of the plane,
// a1, a4).  Here the plane is the exact solution of its 3 x 3 normal
// equations (the problem is linear), and the Gaussian is fitted by
// Levenberg-Marquardt with the analytic Jacobian until the step stalls, in
// FP64; the lanes of a warp share the region's pixels and reduce the normal
// equations in a fixed order, so the fits are deterministic.
#include "sc_common.cuh"

namespace {

constexpr int kSpotWarps = 4;
constexpr int kMaxIter = 200;

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Solves the symmetric positive system A x = b (4 x 4, row-major) by
// Cholesky; false when A is not positive definite.
__device__ bool solve4(const double A[16], const double b[4], double x[4]) {
    double L[16] = {0};
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j <= i; ++j) {
            double s = A[i * 4 + j];
            for (int k = 0; k < j; ++k) s -= L[i * 4 + k] * L[j * 4 + k];
            if (i == j) {
                if (!(s > 0.0)) return false;
                L[i * 4 + i] = sqrt(s);
            } else {
                L[i * 4 + j] = s / L[j * 4 + j];
            }
        }
    double y[4];
    for (int i = 0; i < 4; ++i) {
        double s = b[i];
        for (int k = 0; k < i; ++k) s -= L[i * 4 + k] * y[k];
        y[i] = s / L[i * 4 + i];
    }
    for (int i = 3; i >= 0; --i) {
        double s = y[i];
        for (int k = i + 1; k < 4; ++k) s -= L[k * 4 + i] * x[k];
        x[i] = s / L[i * 4 + i];
    }
    return true;
}

struct Roi {
    const double *img;
    int nh, x0, y0, m, n;
    __device__ double at(int i, int j) const { return img[(size_t)(x0 + i) * nh + (y0 + j)]; }
};

// Cost 0.5 sum r^2 of p over the region (pixel value minus plane d).
__device__ double gauss_cost(const Roi &r, const double *plane, const double p[4], int lane) {
    double c = 0.0;
    for (int k = lane; k < r.m * r.n; k += 32) {
        const int i = k / r.n, j = k - (k / r.n) * r.n;
        const double d = r.at(i, j) - (i * plane[0] + j * plane[1] + plane[2]);
        const double dx = i - p[1], dy = j - p[2];
        const double res = p[0] * exp(-(dx * dx + dy * dy) / p[3]) - d;
        c += res * res;
    }
    return 0.5 * warp_sum_d(c);
}

// out[b] = (center_x, center_y, intensity, background, height, a4, status, 0);
// status 0: a spot; 1: region sum <= 0; 2: plane or fit failed; 3: centre
// outside the region (the reference's skips, spot_detection.py:111-132).
__global__ void __launch_bounds__(kSpotWarps * 32)
spot_fit_kernel(const double *__restrict__ img, int nw, int nh, const double *__restrict__ blobs,
                int n_blobs, double roi_size, double *__restrict__ out) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int b = blockIdx.x * kSpotWarps + warp;
    if (b >= n_blobs) return;
    double *o = out + (size_t)b * 8;
    const double bx = blobs[b * 3], by = blobs[b * 3 + 1];
    // region: int() truncates toward zero as the reference's int() does
    Roi r;
    r.img = img;
    r.nh = nh;
    const int x0 = max(0, (int)(bx - roi_size)), x1 = min(nw, (int)(bx + roi_size) + 1);
    const int y0 = max(0, (int)(by - roi_size)), y1 = min(nh, (int)(by + roi_size) + 1);
    r.x0 = x0;
    r.y0 = y0;
    r.m = x1 - x0;
    r.n = y1 - y0;
    const int m = r.m, n = r.n;
    auto done = [&](double cx, double cy, double inten, double bg, double h, double a4, int st) {
        if (lane == 0) {
            o[0] = cx;
            o[1] = cy;
            o[2] = inten;
            o[3] = bg;
            o[4] = h;
            o[5] = a4;
            o[6] = st;
            o[7] = 0.0;
        }
    };
    if (m <= 0 || n <= 0) {
        done(0, 0, 0, 0, 0, 0, 1);
        return;
    }
    double total = 0.0;
    for (int k = lane; k < m * n; k += 32) total += r.at(k / n, k % n);
    total = warp_sum_d(total);
    if (!(total > 0.0)) {
        done(0, 0, 0, 0, 0, 0, 1);
        return;
    }
    // plane (a5, a6, a7) from the four edges: left row 0 and right row m-1
    // over all j, bottom column 0 and top column n-1 over all i
    double A[6] = {0, 0, 0, 0, 0, 0}, v[3] = {0, 0, 0};  // A: (55, 56, 57, 66, 67, 77)
    auto add = [&](double g0, double g1, double d) {
        A[0] += g0 * g0;
        A[1] += g0 * g1;
        A[2] += g0;
        A[3] += g1 * g1;
        A[4] += g1;
        A[5] += 1.0;
        v[0] += g0 * d;
        v[1] += g1 * d;
        v[2] += d;
    };
    for (int j = lane; j < n; j += 32) {
        add(0.0, j, r.at(0, j));
        add(m - 1, j, r.at(m - 1, j));
    }
    for (int i = lane; i < m; i += 32) {
        add(i, 0.0, r.at(i, 0));
        add(i, n - 1, r.at(i, n - 1));
    }
    for (int q = 0; q < 6; ++q) A[q] = warp_sum_d(A[q]);
    for (int q = 0; q < 3; ++q) v[q] = warp_sum_d(v[q]);
    const double det = A[0] * (A[3] * A[5] - A[4] * A[4]) - A[1] * (A[1] * A[5] - A[4] * A[2]) +
                       A[2] * (A[1] * A[4] - A[3] * A[2]);
    if (!(fabs(det) > 1e-12 * (A[0] * A[3] * A[5] + 1.0))) {
        done(0, 0, 0, 0, 0, 0, 2);
        return;
    }
    double plane[3];
    plane[0] = (v[0] * (A[3] * A[5] - A[4] * A[4]) - A[1] * (v[1] * A[5] - A[4] * v[2]) +
                A[2] * (v[1] * A[4] - A[3] * v[2])) / det;
    plane[1] = (A[0] * (v[1] * A[5] - A[4] * v[2]) - v[0] * (A[1] * A[5] - A[4] * A[2]) +
                A[2] * (A[1] * v[2] - v[1] * A[2])) / det;
    plane[2] = (A[0] * (A[3] * v[2] - v[1] * A[4]) - A[1] * (A[1] * v[2] - v[1] * A[2]) +
                v[0] * (A[1] * A[4] - A[3] * A[2])) / det;
    // sum of the plane over the region; weighted centre of the remainder
    double bg = 0.0, w = 0.0, wx = 0.0, wy = 0.0;
    for (int k = lane; k < m * n; k += 32) {
        const int i = k / n, j = k - (k / n) * n;
        const double pl = i * plane[0] + j * plane[1] + plane[2];
        const double d = r.at(i, j) - pl;
        bg += pl;
        w += d;
        wx += i * d;
        wy += j * d;
    }
    bg = warp_sum_d(bg);
    w = warp_sum_d(w);
    wx = warp_sum_d(wx);
    wy = warp_sum_d(wy);
    double p[4] = {255.0, wx / w, wy / w, roi_size / 2.0};
    double cost = gauss_cost(r, plane, p, lane);
    double lam = 1.0;  // damped first steps: from the reference's start, stay near its minimum
    bool ok = isfinite(cost);
    for (int it = 0; it < kMaxIter && ok; ++it) {
        double H[10] = {0}, g[4] = {0};  // H upper triangle: 00 01 02 03 11 12 13 22 23 33
        for (int k = lane; k < m * n; k += 32) {
            const int i = k / n, j = k - (k / n) * n;
            const double d = r.at(i, j) - (i * plane[0] + j * plane[1] + plane[2]);
            const double dx = i - p[1], dy = j - p[2], r2 = dx * dx + dy * dy;
            const double e = exp(-r2 / p[3]);
            const double res = p[0] * e - d;
            const double J[4] = {e, p[0] * e * 2.0 * dx / p[3], p[0] * e * 2.0 * dy / p[3],
                                 p[0] * e * r2 / (p[3] * p[3])};
            int q = 0;
            for (int a = 0; a < 4; ++a) {
                g[a] += J[a] * res;
                for (int c = a; c < 4; ++c) H[q++] += J[a] * J[c];
            }
        }
        for (int q = 0; q < 10; ++q) H[q] = warp_sum_d(H[q]);
        for (int a = 0; a < 4; ++a) g[a] = warp_sum_d(g[a]);
        // every lane holds the same sums: the step is computed redundantly,
        // with the same result on every lane
        bool stepped = false;
        double step_norm = 0.0, p_norm = 0.0, new_cost = cost;
        for (int tries = 0; tries < 30 && !stepped; ++tries) {
            double M[16];
            int q = 0;
            for (int a = 0; a < 4; ++a)
                for (int c = a; c < 4; ++c) {
                    M[a * 4 + c] = M[c * 4 + a] = H[q];
                    ++q;
                }
            for (int a = 0; a < 4; ++a) M[a * 4 + a] += lam * fmax(M[a * 4 + a], 1e-300);
            const double rhs[4] = {-g[0], -g[1], -g[2], -g[3]};
            double dlt[4];
            if (!solve4(M, rhs, dlt)) {
                lam *= 10.0;
                continue;
            }
            const double pn[4] = {p[0] + dlt[0], p[1] + dlt[1], p[2] + dlt[2], p[3] + dlt[3]};
            const double cn = gauss_cost(r, plane, pn, lane);
            if (isfinite(cn) && cn < cost) {
                step_norm = 0.0;
                p_norm = 0.0;
                for (int a = 0; a < 4; ++a) {
                    step_norm += dlt[a] * dlt[a];
                    p_norm += pn[a] * pn[a];
                    p[a] = pn[a];
                }
                new_cost = cn;
                stepped = true;
                lam = fmax(lam * 0.1, 1e-15);
            } else {
                lam *= 10.0;
            }
        }
        if (!stepped) break;  // no downhill step: a minimum to working precision
        const double drop = cost - new_cost;
        cost = new_cost;
        if (sqrt(step_norm) <= 1e-12 * (sqrt(p_norm) + 1e-12) || drop <= 1e-15 * cost) break;
        ok = isfinite(cost);
    }
    if (!ok || !isfinite(p[0] + p[1] + p[2] + p[3])) {
        done(0, 0, 0, bg, 0, 0, 2);
        return;
    }
    if (!(p[1] >= 0.0 && p[1] < m && p[2] >= 0.0 && p[2] < n)) {
        done(0, 0, 0, bg, p[0], p[3], 3);
        return;
    }
    double inten = 0.0;
    for (int k = lane; k < m * n; k += 32) {
        const int i = k / n, j = k - (k / n) * n;
        const double dx = i - p[1], dy = j - p[2];
        inten += p[0] * exp(-(dx * dx + dy * dy) / p[3]);
    }
    inten = warp_sum_d(inten);
    done(p[1] + x0, p[2] + y0, inten, bg, p[0], p[3], 0);
}

}  // namespace

extern "C" int sc_spot_fit(const double *d_image, int nw, int nh, const double *d_blobs,
                           int n_blobs, double roi_size, double *d_out, void *stream) {
    SC_REQUIRE(nw > 0 && nh > 0 && n_blobs >= 0, "sc_spot_fit: image %dx%d, %d blobs", nw, nh,
               n_blobs);
    SC_REQUIRE(roi_size > 0 && roi_size < 64, "sc_spot_fit: roi_size %g out of (0, 64)", roi_size);
    if (n_blobs == 0) return SC_OK;
    SC_REQUIRE(d_image && d_blobs && d_out, "sc_spot_fit: NULL pointer");
    spot_fit_kernel<<<(n_blobs + kSpotWarps - 1) / kSpotWarps, kSpotWarps * 32, 0,
                      sc::as_stream(stream)>>>(d_image, nw, nh, d_blobs, n_blobs, roi_size, d_out);
    return sc::launch_status("sc_spot_fit");
}
