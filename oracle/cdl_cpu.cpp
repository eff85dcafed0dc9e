// CPU restatement of the CDLmotif CDL ADMM in float32, in the reference's statement
// order, parallel over sequences with OpenMP.
//
// TEST AND MEASUREMENT INFRASTRUCTURE ONLY: the CPU baseline that bench.py times on the
// host cores and that the CPU tests check against the NumPy oracle.  The product
// (libcdlgb.so) never links or calls it.
//
// The reference has no host-array path (its `cdl` struct holds CuArrays,
// src/SETUP/CDL_setup.jl:70-163), so this is the reference's own algorithm written for
// host arrays the way its Julia code would run on them with FFTW: full complex FFTs of
// real arrays promoted to complex, the inverse scaled by 1/Lg and its real part kept,
// every spectrum the reference keeps between iterations kept here too (Y1-hat, Y3-hat,
// d-hat, and the D-step's G2-hat, g1-hat, g2-hat, g3-hat), float32 arithmetic.  FFTW is
// not on this image; the transforms are this file's own mixed-radix Stockham FFT.
//   init (cdl ctor)      src/SETUP/CDL_setup.jl:165-236
//   code_update!         src/CDL/train.jl:1-44, src/CDL/csc_kernels.jl:8-95
//   dict_update!         src/CDL/train.jl:46-89, src/CDL/cdl_kernels.jl:2-77
//   update_best!         src/CDL/train.jl:91-98
//   objective            src/SETUP/CDL_setup.jl:286 (accumulated in float64)
// Layout: a Julia (Lg, M, N) array is [N][M][Lg] here (the same bytes).
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <complex>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

typedef std::complex<float> cf;

// ---------------------------------------------------------------- FFT
// Stockham autosort, decimation in time.  After stage s the data is A[k][j] (k < L =
// product of the radices so far, j < r = n / L): the length-L DFT at frequency k of the
// subsequence x[j], x[j + r], ...  A radix-p stage maps A[k][j' + q r'] (q < p) to
// A'[k + L v][j'] = sum_q w_p^{q v} (w_{Lp}^{q k} A[k][j' + q r']).  Planar (re, im)
// buffers keep the inner loop over j' contiguous.
struct FFTPlan {
    int n = 0;
    std::vector<int> radix;
    std::vector<std::vector<float>> twr, twi;   // per stage: [q][k] twiddles w_{Lp}^{q k}
    std::vector<std::vector<float>> dftr, dfti; // per stage: p x p DFT matrix w_p^{q v}
};

void plan_init(FFTPlan& P, int n) {
    P.n = n;
    int m = n;
    std::vector<int> f;
    for (int p : {4, 2}) while (m % p == 0) { f.push_back(p); m /= p; }
    for (int p = 3; m > 1; p += 2) while (m % p == 0) { f.push_back(p); m /= p; }
    // the largest radix first: its stage has no twiddles (L = 1)
    std::sort(f.begin(), f.end(), [](int a, int b) { return a > b; });
    P.radix = f;
    int L = 1;
    for (int p : f) {
        std::vector<float> tr((size_t)p * L), ti((size_t)p * L), dr((size_t)p * p), di((size_t)p * p);
        for (int q = 0; q < p; ++q)
            for (int k = 0; k < L; ++k) {
                const double a = -2.0 * M_PI * (double)q * k / ((double)L * p);
                tr[(size_t)q * L + k] = (float)cos(a);
                ti[(size_t)q * L + k] = (float)sin(a);
            }
        for (int q = 0; q < p; ++q)
            for (int v = 0; v < p; ++v) {
                const double a = -2.0 * M_PI * (double)((q * v) % p) / p;
                dr[(size_t)q * p + v] = (float)cos(a);
                di[(size_t)q * p + v] = (float)sin(a);
            }
        P.twr.push_back(tr); P.twi.push_back(ti); P.dftr.push_back(dr); P.dfti.push_back(di);
        L *= p;
    }
}

// in: n complex (interleaved); out: n complex; inverse = conjugate twiddles, scaled 1/n.
// work: 6 n floats.
void fft(const FFTPlan& P, const cf* in, cf* out, bool inverse, float* work) {
    const int n = P.n;
    float* ar = work;
    float* ai = work + n;
    float* br = work + 2 * n;
    float* bi = work + 3 * n;
    const float sg = inverse ? -1.f : 1.f;
    for (int i = 0; i < n; ++i) { ar[i] = in[i].real(); ai[i] = sg * in[i].imag(); }
    int L = 1;
    for (size_t s = 0; s < P.radix.size(); ++s) {
        const int p = P.radix[s], r = n / L, rp = r / p;
        const float* twr = P.twr[s].data();
        const float* twi = P.twi[s].data();
        if ((p == 2 || p == 4) && rp < 8) {
            // late stages (few interleaved subsequences): the loops run over k instead
            for (int j = 0; j < rp; ++j) {
                if (p == 2) {
                    const float* __restrict__ w1r = twr + L;
                    const float* __restrict__ w1i = twi + L;
                    for (int k = 0; k < L; ++k) {
                        const size_t xo = (size_t)k * r + j;
                        const float a0r = ar[xo], a0i = ai[xo];
                        const float t1r = ar[xo + rp], t1i = ai[xo + rp];
                        const float a1r = t1r * w1r[k] - t1i * w1i[k], a1i = t1r * w1i[k] + t1i * w1r[k];
                        br[(size_t)k * rp + j] = a0r + a1r; bi[(size_t)k * rp + j] = a0i + a1i;
                        br[(size_t)(k + L) * rp + j] = a0r - a1r; bi[(size_t)(k + L) * rp + j] = a0i - a1i;
                    }
                } else {
                    for (int k = 0; k < L; ++k) {
                        const size_t xo = (size_t)k * r + j;
                        const float w1r = twr[L + k], w1i = twi[L + k];
                        const float w2r = twr[2 * L + k], w2i = twi[2 * L + k];
                        const float w3r = twr[3 * L + k], w3i = twi[3 * L + k];
                        const float a0r = ar[xo], a0i = ai[xo];
                        const float t1r = ar[xo + rp], t1i = ai[xo + rp];
                        const float t2r = ar[xo + 2 * rp], t2i = ai[xo + 2 * rp];
                        const float t3r = ar[xo + 3 * rp], t3i = ai[xo + 3 * rp];
                        const float a1r = t1r * w1r - t1i * w1i, a1i = t1r * w1i + t1i * w1r;
                        const float a2r = t2r * w2r - t2i * w2i, a2i = t2r * w2i + t2i * w2r;
                        const float a3r = t3r * w3r - t3i * w3i, a3i = t3r * w3i + t3i * w3r;
                        const float s02r = a0r + a2r, s02i = a0i + a2i, d02r = a0r - a2r, d02i = a0i - a2i;
                        const float s13r = a1r + a3r, s13i = a1i + a3i, d13r = a1r - a3r, d13i = a1i - a3i;
                        br[(size_t)k * rp + j] = s02r + s13r; bi[(size_t)k * rp + j] = s02i + s13i;
                        br[(size_t)(k + 2 * L) * rp + j] = s02r - s13r; bi[(size_t)(k + 2 * L) * rp + j] = s02i - s13i;
                        br[(size_t)(k + L) * rp + j] = d02r + d13i; bi[(size_t)(k + L) * rp + j] = d02i - d13r;
                        br[(size_t)(k + 3 * L) * rp + j] = d02r - d13i; bi[(size_t)(k + 3 * L) * rp + j] = d02i + d13r;
                    }
                }
            }
            std::swap(ar, br);
            std::swap(ai, bi);
            L *= p;
            continue;
        }
        for (int k = 0; k < L; ++k) {
            const float* xr = ar + (size_t)k * r;
            const float* xi = ai + (size_t)k * r;
            if (p == 2) {
                const float wr = twr[L + k], wi = twi[L + k];
                float* y0r = br + (size_t)k * rp; float* y0i = bi + (size_t)k * rp;
                float* y1r = br + (size_t)(k + L) * rp; float* y1i = bi + (size_t)(k + L) * rp;
                for (int j = 0; j < rp; ++j) {
                    const float a0r = xr[j], a0i = xi[j];
                    const float t1r = xr[j + rp], t1i = xi[j + rp];
                    const float a1r = t1r * wr - t1i * wi, a1i = t1r * wi + t1i * wr;
                    y0r[j] = a0r + a1r; y0i[j] = a0i + a1i;
                    y1r[j] = a0r - a1r; y1i[j] = a0i - a1i;
                }
            } else if (p == 4) {
                const float w1r = twr[L + k], w1i = twi[L + k];
                const float w2r = twr[2 * L + k], w2i = twi[2 * L + k];
                const float w3r = twr[3 * L + k], w3i = twi[3 * L + k];
                float* yr[4]; float* yi[4];
                for (int v = 0; v < 4; ++v) { yr[v] = br + (size_t)(k + L * v) * rp; yi[v] = bi + (size_t)(k + L * v) * rp; }
                for (int j = 0; j < rp; ++j) {
                    const float a0r = xr[j], a0i = xi[j];
                    const float t1r = xr[j + rp], t1i = xi[j + rp];
                    const float t2r = xr[j + 2 * rp], t2i = xi[j + 2 * rp];
                    const float t3r = xr[j + 3 * rp], t3i = xi[j + 3 * rp];
                    const float a1r = t1r * w1r - t1i * w1i, a1i = t1r * w1i + t1i * w1r;
                    const float a2r = t2r * w2r - t2i * w2i, a2i = t2r * w2i + t2i * w2r;
                    const float a3r = t3r * w3r - t3i * w3i, a3i = t3r * w3i + t3i * w3r;
                    const float s02r = a0r + a2r, s02i = a0i + a2i, d02r = a0r - a2r, d02i = a0i - a2i;
                    const float s13r = a1r + a3r, s13i = a1i + a3i, d13r = a1r - a3r, d13i = a1i - a3i;
                    yr[0][j] = s02r + s13r; yi[0][j] = s02i + s13i;
                    yr[2][j] = s02r - s13r; yi[2][j] = s02i - s13i;
                    // w_4 = -i: v = 1 -> d02 - i d13, v = 3 -> d02 + i d13
                    yr[1][j] = d02r + d13i; yi[1][j] = d02i - d13r;
                    yr[3][j] = d02r - d13i; yi[3][j] = d02i + d13r;
                }
            } else {
                // twiddled inputs t[q][j], then out[v][j] = sum_q w_p^{q v} t[q][j]: the
                // loops over j are contiguous (vectorisable)
                const float* dr = P.dftr[s].data();
                const float* di = P.dfti[s].data();
                float* tr_ = work + 4 * n;
                float* ti_ = tr_ + (size_t)p * rp;
                for (int q = 0; q < p; ++q) {
                    const float wr = twr[(size_t)q * L + k], wi = twi[(size_t)q * L + k];
                    const float* vr = xr + (size_t)q * rp;
                    const float* vi = xi + (size_t)q * rp;
                    float* outr = tr_ + (size_t)q * rp;
                    float* outi = ti_ + (size_t)q * rp;
                    for (int j = 0; j < rp; ++j) {
                        outr[j] = vr[j] * wr - vi[j] * wi;
                        outi[j] = vr[j] * wi + vi[j] * wr;
                    }
                }
                // pairs q, p - q: w^{q v} and w^{(p-q) v} are conjugates, so with
                // s_q = t_q + t_{p-q} and d_q = t_q - t_{p-q} the sum over q is
                // t_0 + sum_{q <= (p-1)/2} (Re w^{qv} s_q + i Im w^{qv} d_q)
                const int h = p / 2;
                for (int q = 1; q <= h; ++q) {
                    float* __restrict__ ar_ = tr_ + (size_t)q * rp;
                    float* __restrict__ ai_ = ti_ + (size_t)q * rp;
                    float* __restrict__ cr_ = tr_ + (size_t)(p - q) * rp;
                    float* __restrict__ ci_ = ti_ + (size_t)(p - q) * rp;
                    for (int j = 0; j < rp; ++j) {
                        const float a0 = ar_[j], a1 = ai_[j], c0 = cr_[j], c1 = ci_[j];
                        ar_[j] = a0 + c0; ai_[j] = a1 + c1;      // s_q
                        cr_[j] = a0 - c0; ci_[j] = a1 - c1;      // d_q
                    }
                }
                for (int v = 0; v < p; ++v) {
                    float* __restrict__ yr = br + (size_t)(k + L * v) * rp;
                    float* __restrict__ yi = bi + (size_t)(k + L * v) * rp;
                    const float* __restrict__ t0r = tr_;
                    const float* __restrict__ t0i = ti_;
                    for (int j = 0; j < rp; ++j) { yr[j] = t0r[j]; yi[j] = t0i[j]; }
                    for (int q = 1; q <= h; ++q) {
                        const float cr = dr[(size_t)q * p + v], ci = di[(size_t)q * p + v];
                        const float* __restrict__ sr = tr_ + (size_t)q * rp;
                        const float* __restrict__ si = ti_ + (size_t)q * rp;
                        const float* __restrict__ er = tr_ + (size_t)(p - q) * rp;
                        const float* __restrict__ ei = ti_ + (size_t)(p - q) * rp;
                        // (s + d) w / 2-free form: Re(w) s_q + i Im(w) d_q
                        for (int j = 0; j < rp; ++j) {
                            yr[j] += cr * sr[j] - ci * ei[j];
                            yi[j] += cr * si[j] + ci * er[j];
                        }
                    }
                }
            }
        }
        std::swap(ar, br);
        std::swap(ai, bi);
        L *= p;
    }
    if (inverse) {
        const float sc = 1.f / (float)n;
        for (int i = 0; i < n; ++i) out[i] = cf(ar[i] * sc, -ai[i] * sc);
    } else {
        for (int i = 0; i < n; ++i) out[i] = cf(ar[i], ai[i]);
    }
}

// ---------------------------------------------------------------- state
struct State {
    int N, M, L4, gamma, Lg, flen;
    float rho, sigma, lam, kc, kd;
    FFTPlan plan;
    std::vector<float> S, WtS, diag;
    std::vector<float> X, Y3, y2, y3, X_best;                 // (N, M, Lg)
    std::vector<cf> Y3h;                                       // (N, M, Lg)
    std::vector<float> Y1, y1, DX;                             // (N, Lg)
    std::vector<cf> Y1h;                                       // (N, Lg)
    std::vector<float> d, g1, g3;                              // (N, M, Lg)
    std::vector<cf> dh, g1h, g3h;                              // (N, M, Lg)
    std::vector<float> G2, g2, Td;                             // (N, Lg)
    std::vector<cf> G2h, g2h;                                  // (N, Lg)
    std::vector<float> G1, G3, D_best, dmean;                  // (M, Lg)
    std::vector<cf> G1h, G3h;                                  // (M, Lg)
    double obj_best;
    int nthreads;
};

size_t lmn(const State& s) { return (size_t)s.N * s.M * s.Lg; }

float shrink(float t, float lam) {
    const float a = fabsf(t) - lam;
    const float m = a > 0.f ? a : 0.f;
    return t > 0.f ? m : (t < 0.f ? -m : 0.f);
}

void fft_rows(const State& s, const float* re, cf* out, int rows, std::vector<cf>& tmp, float* work) {
    const int Lg = s.Lg;
    for (int r = 0; r < rows; ++r) {
        for (int l = 0; l < Lg; ++l) tmp[l] = cf(re[(size_t)r * Lg + l], 0.f);
        fft(s.plan, tmp.data(), out + (size_t)r * Lg, false, work);
    }
}

double objective(const State& s) {
    double fit = 0.0, ab = 0.0;
    const size_t L = lmn(s);
#pragma omp parallel for reduction(+ : ab) schedule(static)
    for (long long i = 0; i < (long long)L; ++i) ab += fabs((double)s.X[i]);
    for (int n = 0; n < s.N; ++n)
        for (int j = 0; j < s.L4; ++j) {
            const double r = (double)s.DX[(size_t)n * s.Lg + s.gamma + j] - (double)s.S[(size_t)n * s.L4 + j];
            fit += r * r;
        }
    return 0.5 * fit + (double)s.lam * ab;
}

// code_update!: all num_iter X-steps of one sequence (they couple only its M filters)
void code_update_seq(State& s, int n, int iters, const std::vector<cf>& At, std::vector<cf>& tmp,
                     std::vector<cf>& Y2h, std::vector<cf>& y2h, std::vector<cf>& y3h,
                     std::vector<cf>& RHS, std::vector<cf>& y1h, std::vector<cf>& alpha,
                     float* work) {
    const int M = s.M, Lg = s.Lg;
    const size_t o = (size_t)n * M * Lg, ol = (size_t)n * Lg;
    float* X = &s.X[o]; float* y2 = &s.y2[o]; float* y3 = &s.y3[o]; float* Y3 = &s.Y3[o];
    cf* Y3h = &s.Y3h[o];
    float* Y1 = &s.Y1[ol]; float* y1 = &s.y1[ol]; float* DX = &s.DX[ol];
    cf* Y1h = &s.Y1h[ol];
    std::vector<float> Y2((size_t)M * Lg);
    const cf* G1h = s.G1h.data();
    for (int it = 0; it < iters; ++it) {
        for (size_t i = 0; i < (size_t)M * Lg; ++i) Y2[i] = shrink(X[i] + y2[i], s.lam);   // :7
        fft_rows(s, Y2.data(), Y2h.data(), M, tmp, work);                                 // :8
        for (int l = 0; l < Lg; ++l) y1[l] = y1[l] + DX[l] - Y1[l];                       // :12
        fft_rows(s, y1, y1h.data(), 1, tmp, work);
        for (size_t i = 0; i < (size_t)M * Lg; ++i) y2[i] = y2[i] + X[i] - Y2[i];         // :13
        fft_rows(s, y2, y2h.data(), M, tmp, work);
        for (size_t i = 0; i < (size_t)M * Lg; ++i) y3[i] = y3[i] + X[i] - Y3[i];         // :14
        fft_rows(s, y3, y3h.data(), M, tmp, work);
        // sherman_CSC_RHS! (:21-23)
        for (int m = 0; m < M; ++m)
            for (int l = 0; l < Lg; ++l) {
                const size_t i = (size_t)m * Lg + l;
                RHS[i] = std::conj(G1h[i]) * (Y1h[l] - y1h[l]) + (Y2h[i] - y2h[i]) + (Y3h[i] - y3h[i]);
            }
        // sherman_CSC_dot! (:24): alpha = sum_m At .* RHS (serial over m)
        for (int l = 0; l < Lg; ++l) alpha[l] = cf(0.f, 0.f);
        for (int m = 0; m < M; ++m)
            for (int l = 0; l < Lg; ++l) alpha[l] += At[(size_t)m * Lg + l] * RHS[(size_t)m * Lg + l];
        // sherman_CSC_combine! (:25): Xh = (RHS - alpha conj(G1h)) / k (in RHS)
        for (int m = 0; m < M; ++m)
            for (int l = 0; l < Lg; ++l) {
                const size_t i = (size_t)m * Lg + l;
                RHS[i] = (RHS[i] - alpha[l] * std::conj(G1h[i])) / s.kc;
            }
        // X = real(ifft(Xh)) (:26), DX = real(ifft(sum_m G1h Xh)) (:27)
        for (int m = 0; m < M; ++m) {
            fft(s.plan, &RHS[(size_t)m * Lg], tmp.data(), true, work);
            for (int l = 0; l < Lg; ++l) X[(size_t)m * Lg + l] = tmp[l].real();
        }
        for (int l = 0; l < Lg; ++l) alpha[l] = cf(0.f, 0.f);
        for (int m = 0; m < M; ++m)
            for (int l = 0; l < Lg; ++l) alpha[l] += G1h[(size_t)m * Lg + l] * RHS[(size_t)m * Lg + l];
        fft(s.plan, alpha.data(), tmp.data(), true, work);
        for (int l = 0; l < Lg; ++l) DX[l] = tmp[l].real();
        // update_Y1! (:35), Y1-hat (:36)
        for (int l = 0; l < Lg; ++l)
            Y1[l] = (s.WtS[ol + l] + s.rho * (DX[l] + y1[l])) / (s.diag[l] + s.rho);
        fft_rows(s, Y1, Y1h, 1, tmp, work);
        // projectionX! (:40), Y3-hat (:41)
        for (int m = 0; m < M; ++m)
            for (int l = 0; l < Lg; ++l) {
                const size_t i = (size_t)m * Lg + l;
                Y3[i] = (l % 4 == 0) ? X[i] + y3[i] : 0.f;
            }
        fft_rows(s, Y3, Y3h, M, tmp, work);
    }
}

void code_update(State& s, int iters) {
    const int M = s.M, Lg = s.Lg;
    // a = G1-hat; At = a ./ (sum_m |a|^2 + k) (train.jl:18-20)
    std::vector<float> sd(Lg, 0.f);
    for (int m = 0; m < M; ++m)
        for (int l = 0; l < Lg; ++l) sd[l] += std::norm(s.G1h[(size_t)m * Lg + l]);
    std::vector<cf> At((size_t)M * Lg);
    for (int m = 0; m < M; ++m)
        for (int l = 0; l < Lg; ++l) At[(size_t)m * Lg + l] = s.G1h[(size_t)m * Lg + l] / (sd[l] + s.kc);
#pragma omp parallel
    {
        std::vector<cf> tmp(Lg), Y2h((size_t)M * Lg), y2h((size_t)M * Lg), y3h((size_t)M * Lg),
            RHS((size_t)M * Lg), y1h(Lg), alpha(Lg);
        std::vector<float> work(6 * (size_t)Lg);
#pragma omp for schedule(dynamic, 4)
        for (int n = 0; n < s.N; ++n)
            code_update_seq(s, n, iters, At, tmp, Y2h, y2h, y3h, RHS, y1h, alpha, work.data());
    }
}

void project_G(State& s, const std::vector<float>& v1, const std::vector<float>& v2) {
    const int M = s.M, Lg = s.Lg, flen = s.flen;
    // projection2box! (cdl_kernels.jl:37-51)
    for (int m = 0; m < M; ++m)
        for (int l = 0; l < Lg; ++l) {
            const float b = v2[(size_t)m * Lg + l];
            const bool sup = l < flen;
            s.G3[(size_t)m * Lg + l] = b >= 1.f ? (sup ? 1.f : 0.f) : (b <= 0.f ? 0.f : (sup ? b : 0.f));
        }
    // prox_simplex_zeros! with the reference's group index (cdl_kernels.jl:53-66)
    for (int m = 0; m < M; ++m)
        for (int l = 0; l < Lg; ++l) {
            float out = 0.f;
            if (l < flen) {
                const int i = 4 * ((l + 1) / 4);
                const float* v = &v1[(size_t)m * Lg];
                const float grp = v[i] + v[i + 1] + v[i + 2] + v[i + 3];
                out = v[l] - 0.25f * (grp - 1.f);
            }
            s.G1[(size_t)m * Lg + l] = out;
        }
}

void dict_update(State& s, int iters) {
    const int M = s.M, Lg = s.Lg, N = s.N;
    const size_t LM = (size_t)M * Lg;
    for (int it = 0; it < iters; ++it) {
        int nt = 1;
#ifdef _OPENMP
        nt = omp_get_max_threads();
#endif
        std::vector<double> part1((size_t)nt * LM, 0.0), part3((size_t)nt * LM, 0.0),
            partd((size_t)nt * LM, 0.0);
        const cf* G1h = s.G1h.data();
        const cf* G3h = s.G3h.data();
#pragma omp parallel
        {
            int tid = 0;
#ifdef _OPENMP
            tid = omp_get_thread_num();
#endif
            double* p1 = &part1[(size_t)tid * LM];
            double* p3 = &part3[(size_t)tid * LM];
            double* pd = &partd[(size_t)tid * LM];
            std::vector<cf> tmp(Lg), RHS(LM), T(Lg), beta(Lg);
            std::vector<float> sdots(Lg), work(6 * (size_t)Lg);
#pragma omp for schedule(static)
            for (int n = 0; n < N; ++n) {
                const size_t o = (size_t)n * LM, ol = (size_t)n * Lg;
                const cf* Y3h = &s.Y3h[o];
                cf* dh = &s.dh[o];
                // sum_dots = sum_m |Y3-hat|^2 + k; X_cdl = Y3-hat / sum_dots (:52-54)
                for (int l = 0; l < Lg; ++l) sdots[l] = 0.f;
                for (int m = 0; m < M; ++m)
                    for (int l = 0; l < Lg; ++l) sdots[l] += std::norm(Y3h[(size_t)m * Lg + l]);
                // Td = real(ifft(sum_m Y3-hat d-hat_old)) (:56-57)
                for (int l = 0; l < Lg; ++l) T[l] = cf(0.f, 0.f);
                for (int m = 0; m < M; ++m)
                    for (int l = 0; l < Lg; ++l) T[l] += Y3h[(size_t)m * Lg + l] * dh[(size_t)m * Lg + l];
                fft(s.plan, T.data(), tmp.data(), true, work.data());
                for (int l = 0; l < Lg; ++l) s.Td[ol + l] = tmp[l].real();
                // sherman_CDL_RHS! (:58)
                for (int m = 0; m < M; ++m)
                    for (int l = 0; l < Lg; ++l) {
                        const size_t i = (size_t)m * Lg + l;
                        RHS[i] = std::conj(Y3h[i]) * (s.G2h[ol + l] - s.g2h[ol + l]) +
                                 (G1h[i] - s.g1h[o + i]) + (G3h[i] - s.g3h[o + i]);
                    }
                // beta = sum_m X_cdl RHS (:59); d-hat = RHS - beta conj(Y3-hat) (:60, no 1/2)
                for (int l = 0; l < Lg; ++l) beta[l] = cf(0.f, 0.f);
                for (int m = 0; m < M; ++m)
                    for (int l = 0; l < Lg; ++l) {
                        const size_t i = (size_t)m * Lg + l;
                        beta[l] += (Y3h[i] / (sdots[l] + s.kd)) * RHS[i];
                    }
                for (int m = 0; m < M; ++m)
                    for (int l = 0; l < Lg; ++l) {
                        const size_t i = (size_t)m * Lg + l;
                        dh[i] = RHS[i] - beta[l] * std::conj(Y3h[i]);
                    }
                // d = real(ifft(d-hat)) (:61)
                float* d = &s.d[o];
                for (int m = 0; m < M; ++m) {
                    fft(s.plan, &dh[(size_t)m * Lg], tmp.data(), true, work.data());
                    for (int l = 0; l < Lg; ++l) d[(size_t)m * Lg + l] = tmp[l].real();
                }
                // update_g2! (:68), G2-hat (:69); g2 += Td - G2 (:71)
                for (int l = 0; l < Lg; ++l)
                    s.G2[ol + l] = (s.WtS[ol + l] + s.sigma * (s.Td[ol + l] + s.g2[ol + l])) / (s.diag[l] + s.sigma);
                fft_rows(s, &s.G2[ol], &s.G2h[ol], 1, tmp, work.data());
                // g1 += d - G1 (:70), g3 += d - G3 (:72), their spectra
                float* g1 = &s.g1[o];
                float* g3 = &s.g3[o];
                for (size_t i = 0; i < LM; ++i) {
                    g1[i] = g1[i] + d[i] - s.G1[i];
                    g3[i] = g3[i] + d[i] - s.G3[i];
                }
                fft_rows(s, g1, &s.g1h[o], M, tmp, work.data());
                for (int l = 0; l < Lg; ++l) s.g2[ol + l] = s.g2[ol + l] + s.Td[ol + l] - s.G2[ol + l];
                fft_rows(s, &s.g2[ol], &s.g2h[ol], 1, tmp, work.data());
                fft_rows(s, g3, &s.g3h[o], M, tmp, work.data());
                // the consensus sums (:76, :83) and D_best's (:95), per thread
                for (size_t i = 0; i < LM; ++i) {
                    p1[i] += (double)(d[i] + g1[i]);
                    p3[i] += (double)(d[i] + g3[i]);
                    pd[i] += (double)d[i];
                }
            }
        }
        // thread partials in a fixed order, then the means in float32
        std::vector<float> v1(LM), v2(LM);
        for (size_t i = 0; i < LM; ++i) {
            double a = 0, b = 0, c = 0;
            for (int t = 0; t < nt; ++t) { a += part1[(size_t)t * LM + i]; b += part3[(size_t)t * LM + i]; c += partd[(size_t)t * LM + i]; }
            v1[i] = (float)(a / N);
            v2[i] = (float)(b / N);
            s.dmean[i] = (float)(c / N);
        }
        project_G(s, v1, v2);
        std::vector<cf> tmp(Lg);
        std::vector<float> work(6 * (size_t)Lg);
        fft_rows(s, s.G3.data(), s.G3h.data(), M, tmp, work.data());          // :78
        fft_rows(s, s.G1.data(), s.G1h.data(), M, tmp, work.data());          // :85
    }
}

double update_best(State& s, int* improved) {
    const double obj = objective(s);
    *improved = obj < s.obj_best;
    if (*improved) {
        s.obj_best = obj;
        s.D_best = s.dmean;
        s.X_best = s.X;
    }
    return obj;
}

}  // namespace

extern "C" {

// S (N, 4L) one-hot, X0 (N, M, Lg), D0 (M, Lg); returns an opaque state or NULL.
void* cdlcpu_create(const float* S, const float* X0, const float* D0, int N, int L4, int M,
                    int filter_size, float rho, float sigma, float lam, int nthreads) {
    State* s = new State();
    s->N = N; s->M = M; s->L4 = L4; s->gamma = 4 * filter_size; s->flen = 4 * filter_size;
    s->Lg = L4 + 2 * s->gamma;
    s->rho = rho; s->sigma = sigma; s->lam = lam; s->kc = 2.f; s->kd = 2.f;
    s->nthreads = nthreads;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
    const int Lg = s->Lg;
    const size_t LMN = (size_t)N * M * Lg, LN = (size_t)N * Lg, LM = (size_t)M * Lg;
    plan_init(s->plan, Lg);
    for (int p : s->plan.radix)
        if (p > 64) { delete s; return nullptr; }    // the generic butterfly holds 64 points
    s->S.assign(S, S + (size_t)N * L4);
    s->diag.assign(Lg, 0.f);
    for (int l = s->gamma; l < s->gamma + L4; ++l) s->diag[l] = 1.f;
    s->WtS.assign(LN, 0.f);
    for (int n = 0; n < N; ++n)
        for (int j = 0; j < L4; ++j) s->WtS[(size_t)n * Lg + s->gamma + j] = S[(size_t)n * L4 + j];
    // D0 masked by P_D, X0 by enforce_dummy_code_constraint! (CDL_setup.jl:183, 191-192)
    std::vector<float> D(LM, 0.f);
    for (int m = 0; m < M; ++m)
        for (int l = 0; l < s->flen; ++l) D[(size_t)m * Lg + l] = D0[(size_t)m * Lg + l];
    s->X.assign(LMN, 0.f);
    for (size_t i = 0; i < LMN; ++i) s->X[i] = (i % Lg) % 4 == 0 ? X0[i] : 0.f;
    s->G1 = D; s->G3 = D; s->D_best = D; s->dmean = D;
    s->G1h.resize(LM); s->G3h.resize(LM);
    std::vector<cf> tmp(Lg), Dh(LM);
    std::vector<float> work(6 * (size_t)Lg);
    fft_rows(*s, D.data(), Dh.data(), M, tmp, work.data());
    s->G1h = Dh; s->G3h = Dh;
    s->Y3 = s->X;  s->X_best = s->X;
    s->y2.assign(LMN, 0.f); s->y3.assign(LMN, 0.f);
    s->g1.assign(LMN, 0.f); s->g3.assign(LMN, 0.f);
    s->d.resize(LMN); s->dh.resize(LMN); s->Y3h.resize(LMN);
    s->g1h.assign(LMN, cf(0.f, 0.f)); s->g3h.assign(LMN, cf(0.f, 0.f));
    s->Y1.assign(LN, 0.f); s->y1.assign(LN, 0.f); s->DX.assign(LN, 0.f);
    s->Y1h.assign(LN, cf(0.f, 0.f));
    s->g2.assign(LN, 0.f); s->Td.assign(LN, 0.f); s->G2.resize(LN); s->G2h.resize(LN);
    s->g2h.assign(LN, cf(0.f, 0.f));
    std::vector<float> dcol(Lg);
    for (int m = 0; m < M; ++m) {
        fft(s->plan, &Dh[(size_t)m * Lg], tmp.data(), true, work.data());
        for (int l = 0; l < Lg; ++l) dcol[l] = tmp[l].real();
        for (int n = 0; n < N; ++n) {
            memcpy(&s->d[(size_t)n * LM + (size_t)m * Lg], dcol.data(), Lg * 4);
            memcpy(&s->dh[(size_t)n * LM + (size_t)m * Lg], &Dh[(size_t)m * Lg], Lg * sizeof(cf));
        }
    }
    // DX = real(ifft(sum_m D-hat X-hat)), G2 = DX, Y3-hat = X-hat (CDL_setup.jl:197-230)
#pragma omp parallel
    {
        std::vector<cf> t2(Lg), acc(Lg), Xh((size_t)M * Lg);
        std::vector<float> w2(6 * (size_t)Lg);
#pragma omp for schedule(static)
        for (int n = 0; n < N; ++n) {
            const size_t o = (size_t)n * LM;
            fft_rows(*s, &s->X[o], Xh.data(), M, t2, w2.data());
            memcpy(&s->Y3h[o], Xh.data(), LM * sizeof(cf));
            for (int l = 0; l < Lg; ++l) acc[l] = cf(0.f, 0.f);
            for (int m = 0; m < M; ++m)
                for (int l = 0; l < Lg; ++l) acc[l] += Dh[(size_t)m * Lg + l] * Xh[(size_t)m * Lg + l];
            fft(s->plan, acc.data(), t2.data(), true, w2.data());
            for (int l = 0; l < Lg; ++l) s->DX[(size_t)n * Lg + l] = t2[l].real();
            fft_rows(*s, &s->DX[(size_t)n * Lg], &s->G2h[(size_t)n * Lg], 1, t2, w2.data());
        }
    }
    s->G2 = s->DX;
    s->obj_best = objective(*s);
    return s;
}

void cdlcpu_destroy(void* h) { delete (State*)h; }

double cdlcpu_obj_best(void* h) { return ((State*)h)->obj_best; }

// iter_num passes of cdl_optimize's loop body (wrap.jl:6-11); objs: iter_num values
void cdlcpu_run_outer(void* h, int iter_num, int csc_iter, int cdl_iter, double* objs) {
    State* s = (State*)h;
#ifdef _OPENMP
    if (s->nthreads > 0) omp_set_num_threads(s->nthreads);
#endif
    for (int it = 0; it < iter_num; ++it) {
        code_update(*s, csc_iter);
        int imp = 0;
        const double o = update_best(*s, &imp);
        dict_update(*s, cdl_iter);
        if (objs) objs[it] = o;
    }
}

// copy a field out: 0 X, 1 d, 2 G1, 3 D_best, 4 DX, 5 X_best, 6 G3
int cdlcpu_get(void* h, int field, float* dst) {
    State* s = (State*)h;
    const std::vector<float>* v = nullptr;
    switch (field) {
        case 0: v = &s->X; break;
        case 1: v = &s->d; break;
        case 2: v = &s->G1; break;
        case 3: v = &s->D_best; break;
        case 4: v = &s->DX; break;
        case 5: v = &s->X_best; break;
        case 6: v = &s->G3; break;
        default: return -1;
    }
    memcpy(dst, v->data(), v->size() * sizeof(float));
    return 0;
}

int cdlcpu_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

}  // extern "C"
