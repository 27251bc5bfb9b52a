// Host side of the masked-basin inversion: the land boundary B and the inverse FP64
// capacitance matrices, one per vertical mode.
//
// The DST-I solve G = (lap - lam)^-1 acts on the full (Ny, Nx) array with zeros outside it.
// For a member with interior land, psi must vanish on B (land cells with an interior ocean
// cell among their 8 neighbours: every cell the ocean's stencils reach).  The
// capacitance-matrix method (Thiry et al. 2024) does that with a second solve:
//   psi1 = G rhs,  sigma = -C^-1 psi1[B],  psi = G (rhs + E_B sigma),  C = G[B, B].
// C is built here in FP64 from the separable structure of G: with Sx the orthonormal DST-I
// matrix along x and ex its eigenvalues,
//   G[(y, x), (y', x')] = sum_kx Sx[x, kx] Sx[x', kx] H_kx[y, y'],
//   H_kx = (Dyy + (ex[kx] - lam) I)^-1,
// Dyy the 3-point second difference along y with zeros outside the array.  The columns of the
// tridiagonal inverse H_kx come from the Thomas algorithm, so C costs O(Nx k^2) instead of a
// solve per boundary point.  -C is symmetric positive definite (lap - lam is negative
// definite for lam >= 0): C^-1 = -(L L^T)^-1 from a blocked Cholesky factorisation.  All loops
// over rows run on every host thread.
#include <algorithm>
#include <cmath>
#include <thread>
#include <vector>

#include "qg_internal.cuh"

namespace qg {

namespace {

template <typename F>
void parallel_for(int n, F&& f) {
    const int nt = std::max(1, std::min<int>(n, (int)std::thread::hardware_concurrency()));
    if (nt == 1 || n < 64) {
        for (int i = 0; i < n; ++i) f(i);
        return;
    }
    std::vector<std::thread> th;
    for (int t = 0; t < nt; ++t)
        th.emplace_back([&, t] {
            for (int i = t; i < n; i += nt) f(i);
        });
    for (auto& x : th) x.join();
}

// In place: A (n x n, row-major, SPD) -> its lower Cholesky factor in the lower triangle.
// Returns false if a pivot is not positive.
bool cholesky(std::vector<double>& A, int n) {
    constexpr int NB = 64;
    for (int j0 = 0; j0 < n; j0 += NB) {
        const int j1 = std::min(n, j0 + NB);
        // diagonal block
        for (int j = j0; j < j1; ++j) {
            double d = A[(size_t)j * n + j];
            for (int k = j0; k < j; ++k) d -= A[(size_t)j * n + k] * A[(size_t)j * n + k];
            if (!(d > 0.0)) return false;
            d = std::sqrt(d);
            A[(size_t)j * n + j] = d;
            for (int i = j + 1; i < j1; ++i) {
                double s = A[(size_t)i * n + j];
                for (int k = j0; k < j; ++k) s -= A[(size_t)i * n + k] * A[(size_t)j * n + k];
                A[(size_t)i * n + j] = s / d;
            }
        }
        // panel below the block: rows i >= j1, columns j0..j1-1 (triangular solve)
        parallel_for(n - j1, [&](int r) {
            const int i = j1 + r;
            double* Ai = &A[(size_t)i * n];
            for (int j = j0; j < j1; ++j) {
                double s = Ai[j];
                const double* Aj = &A[(size_t)j * n];
                for (int k = j0; k < j; ++k) s -= Ai[k] * Aj[k];
                Ai[j] = s / Aj[j];
            }
        });
        // trailing update of the lower triangle: A[i][j] -= sum_k A[i][k] A[j][k]
        parallel_for(n - j1, [&](int r) {
            const int i = j1 + r;
            double* Ai = &A[(size_t)i * n];
            for (int j = j1; j <= i; ++j) {
                const double* Aj = &A[(size_t)j * n];
                double s = 0.0;
                for (int k = j0; k < j1; ++k) s += Ai[k] * Aj[k];
                Ai[j] -= s;
            }
        });
    }
    return true;
}

// X = (L L^T)^-1 = W^T W with W = L^-1, from the lower factor in A (full symmetric X,
// row-major).  Columns of W by forward substitution (row-wise reads of L), stored as rows.
void cholesky_inverse(const std::vector<double>& A, int n, std::vector<double>& X) {
    std::vector<double> Wc((size_t)n * n, 0.0);  // Wc[c][k] = W[k][c], zero for k < c
    parallel_for(n, [&](int c) {
        double* y = &Wc[(size_t)c * n];
        for (int i = c; i < n; ++i) {
            double s = (i == c) ? 1.0 : 0.0;
            const double* Ai = &A[(size_t)i * n];
            for (int k = c; k < i; ++k) s -= Ai[k] * y[k];
            y[i] = s / Ai[i];
        }
    });
    X.assign((size_t)n * n, 0.0);
    parallel_for(n, [&](int i) {
        const double* wi = &Wc[(size_t)i * n];
        for (int j = 0; j <= i; ++j) {
            const double* wj = &Wc[(size_t)j * n];
            double s = 0.0;
            for (int k = i; k < n; ++k) s += wi[k] * wj[k];  // k >= max(i, j) = i
            X[(size_t)i * n + j] = s;
        }
    });
    for (int i = 0; i < n; ++i)
        for (int j = i + 1; j < n; ++j) X[(size_t)i * n + j] = X[(size_t)j * n + i];
}

}  // namespace

// B of a masked member (linear indices j * Nx + i, ascending).
std::vector<int> land_boundary(const qg_member_desc& d) {
    const int Ny = d.ny + 2, Nx = d.nx + 2;
    std::vector<int> out;
    if (!d.mask) return out;
    auto land = [&](int j, int i) {
        return j > 0 && i > 0 && j < Ny - 1 && i < Nx - 1 && d.mask[(size_t)j * Nx + i] == 0;
    };
    auto ocean = [&](int j, int i) {
        return j > 0 && i > 0 && j < Ny - 1 && i < Nx - 1 && d.mask[(size_t)j * Nx + i] != 0;
    };
    for (int j = 1; j < Ny - 1; ++j)
        for (int i = 1; i < Nx - 1; ++i) {
            if (!land(j, i)) continue;
            bool near = false;
            for (int dj = -1; dj <= 1 && !near; ++dj)
                for (int di = -1; di <= 1 && !near; ++di)
                    if ((dj || di) && ocean(j + dj, i + di)) near = true;
            if (near) out.push_back(j * Nx + i);
        }
    return out;
}

// Inverse capacitance matrices C_m^-1 (nl x k x k, row-major) of a masked member for the
// Helmholtz lambdas lam[0..nl-1].  Returns false if a factorisation fails.
bool capacitance_inverse(const qg_member_desc& d, const double* lam, int nl, const std::vector<int>& B,
                         std::vector<double>& cinv) {
    const int Ny = d.ny + 2, Nx = d.nx + 2, k = (int)B.size();
    const double dx = d.Lx / d.nx, dy = d.Ly / d.ny;
    cinv.assign((size_t)nl * k * k, 0.0);
    if (k == 0) return true;
    std::vector<int> bx(k), by(k);
    for (int p = 0; p < k; ++p) {
        by[p] = B[p] / Nx;
        bx[p] = B[p] % Nx;
    }
    // distinct rows of B and each point's index among them
    std::vector<int> ys(by);
    std::sort(ys.begin(), ys.end());
    ys.erase(std::unique(ys.begin(), ys.end()), ys.end());
    const int ny_b = (int)ys.size();
    std::vector<int> yi(k);
    for (int p = 0; p < k; ++p) yi[p] = (int)(std::lower_bound(ys.begin(), ys.end(), by[p]) - ys.begin());
    // Sx at the boundary points, by kx: SB[q][p] = Sx[bx[p], q]
    const double sx = std::sqrt(2.0 / (Nx + 1));
    std::vector<double> SB((size_t)Nx * k);
    parallel_for(Nx, [&](int q) {
        const long long per = 2LL * (Nx + 1);  // argument reduced for accuracy
        for (int p = 0; p < k; ++p)
            SB[(size_t)q * k + p] = sx * std::sin(M_PI * (double)(((long long)(bx[p] + 1) * (q + 1)) % per) / (Nx + 1));
    });
    std::vector<double> ex(Nx);
    for (int q = 0; q < Nx; ++q) {
        const double sn = std::sin(M_PI * (q + 1) / (2.0 * (Nx + 1)));
        ex[q] = -4.0 * sn * sn / (dx * dx);
    }
    std::vector<double> C((size_t)k * k);
    constexpr int QC = 16;  // kx per chunk: the chunk's H matrices stay small
    std::vector<double> Hs((size_t)QC * ny_b * ny_b);
    for (int m = 0; m < nl; ++m) {
        std::fill(C.begin(), C.end(), 0.0);
        for (int q0 = 0; q0 < Nx; q0 += QC) {
            const int nq = std::min(QC, Nx - q0);
            // H_kx restricted to the rows of B, by the Thomas algorithm (diagonally dominant)
            parallel_for(nq * ny_b, [&](int t) {
                const int qq = t / ny_b, c = t % ny_b, q = q0 + qq;
                const double off = 1.0 / (dy * dy), diag = -2.0 / (dy * dy) + ex[q] - lam[m];
                std::vector<double> den(Ny), cp(Ny), h(Ny);
                den[0] = diag;
                for (int j = 1; j < Ny; ++j) den[j] = diag - off * off / den[j - 1];
                const int y0 = ys[c];
                for (int j = 0; j < Ny; ++j)
                    cp[j] = (j == y0 ? 1.0 : 0.0) - (j > 0 ? off * cp[j - 1] / den[j - 1] : 0.0);
                h[Ny - 1] = cp[Ny - 1] / den[Ny - 1];
                for (int j = Ny - 2; j >= 0; --j) h[j] = (cp[j] - off * h[j + 1]) / den[j];
                double* H = &Hs[(size_t)qq * ny_b * ny_b];
                for (int r = 0; r < ny_b; ++r) H[(size_t)r * ny_b + c] = h[ys[r]];
            });
            // C[p][r] += sum over the chunk of Sx[bx_p] Sx[bx_r] H[by_p][by_r] (lower triangle)
            parallel_for(k, [&](int p) {
                double* Cp = &C[(size_t)p * k];
                for (int qq = 0; qq < nq; ++qq) {
                    const double* S = &SB[(size_t)(q0 + qq) * k];
                    const double sp = S[p];
                    const double* H = &Hs[(size_t)qq * ny_b * ny_b + (size_t)yi[p] * ny_b];
                    for (int r = 0; r <= p; ++r) Cp[r] += sp * S[r] * H[yi[r]];
                }
            });
        }
        // A = -C (lower triangle), Cholesky, inverse; C^-1 = -A^-1
        std::vector<double> A((size_t)k * k);
        for (int p = 0; p < k; ++p)
            for (int r = 0; r <= p; ++r) A[(size_t)p * k + r] = -C[(size_t)p * k + r];
        if (!cholesky(A, k)) return false;
        std::vector<double> X;
        cholesky_inverse(A, k, X);
        double* out = &cinv[(size_t)m * k * k];
        for (size_t t = 0; t < (size_t)k * k; ++t) out[t] = -X[t];
    }
    return true;
}

}  // namespace qg
