// The transforms behind oracle/ref_fftw/fftw3.h: 2-D complex DFTs and batched 2-D
// real-to-complex / complex-to-real DFTs with FFTW's conventions, computed in double
// precision (radix-2 FFT for power-of-two lengths, the direct sum otherwise) and rounded
// to float once per output.  Test infrastructure: it lets emsim's FFTW extension run
// unchanged where libfftw3f is absent; results agree with FFTW's float transforms to
// float rounding, which is what the golden vectors made with it are compared at.
#include <cmath>
#include <complex>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "fftw3.h"

namespace {

using cd = std::complex<double>;

enum Kind { C2C, R2C, C2R };

// in-place 1-D DFT of x (length n, stride 1); sign -1 forward, +1 backward
void dft1(std::vector<cd>& x, int sign) {
    const size_t n = x.size();
    if (n <= 1) return;
    if ((n & (n - 1)) == 0) {
        for (size_t i = 1, j = 0; i < n; ++i) {  // bit reversal
            size_t bit = n >> 1;
            for (; j & bit; bit >>= 1) j ^= bit;
            j ^= bit;
            if (i < j) std::swap(x[i], x[j]);
        }
        for (size_t len = 2; len <= n; len <<= 1) {
            for (size_t i = 0; i < n; i += len) {
                for (size_t k = 0; k < len / 2; ++k) {
                    const double a = sign * 2.0 * M_PI * (double)k / (double)len;
                    const cd w(std::cos(a), std::sin(a));
                    const cd u = x[i + k], v = x[i + k + len / 2] * w;
                    x[i + k] = u + v;
                    x[i + k + len / 2] = u - v;
                }
            }
        }
        return;
    }
    std::vector<cd> y(n);
    for (size_t k = 0; k < n; ++k) {
        cd s = 0.0;
        for (size_t j = 0; j < n; ++j) {
            const double a = sign * 2.0 * M_PI * (double)((j * k) % n) / (double)n;
            s += x[j] * cd(std::cos(a), std::sin(a));
        }
        y[k] = s;
    }
    x.swap(y);
}

// 2-D transform of an n0 x m array (row-major) along both dimensions
void dft2(std::vector<cd>& a, int n0, int m, int sign, bool rows = true, bool cols = true) {
    std::vector<cd> line;
    if (rows) {
        line.resize(m);
        for (int i = 0; i < n0; ++i) {
            for (int j = 0; j < m; ++j) line[j] = a[(size_t)i * m + j];
            dft1(line, sign);
            for (int j = 0; j < m; ++j) a[(size_t)i * m + j] = line[j];
        }
    }
    if (cols) {
        line.resize(n0);
        for (int j = 0; j < m; ++j) {
            for (int i = 0; i < n0; ++i) line[i] = a[(size_t)i * m + j];
            dft1(line, sign);
            for (int i = 0; i < n0; ++i) a[(size_t)i * m + j] = line[i];
        }
    }
}

}  // namespace

struct fftwf_plan_s {
    Kind kind;
    int n0, n1, sign, howmany, idist, odist;
    float* rin;
    fftwf_complex* cin;
    fftwf_complex* cout;
    float* rout;
};

extern "C" {

int fftwf_init_threads(void) { return 1; }
void fftwf_plan_with_nthreads(int) {}
void* fftwf_malloc(size_t n) { return std::malloc(n); }
void fftwf_free(void* p) { std::free(p); }
void fftwf_destroy_plan(fftwf_plan p) { delete p; }

fftwf_plan fftwf_plan_dft_2d(int n0, int n1, fftwf_complex* in, fftwf_complex* out, int sign, unsigned) {
    return new fftwf_plan_s{C2C, n0, n1, sign, 1, n0 * n1, n0 * n1, nullptr, in, out, nullptr};
}

fftwf_plan fftwf_plan_many_dft_r2c(int rank, const int* n, int howmany, float* in, const int*, int istride,
                                   int idist, fftwf_complex* out, const int*, int ostride, int odist, unsigned) {
    if (rank != 2 || istride != 1 || ostride != 1) std::abort();
    return new fftwf_plan_s{R2C, n[0], n[1], FFTW_FORWARD, howmany, idist, odist, in, nullptr, out, nullptr};
}

fftwf_plan fftwf_plan_many_dft_c2r(int rank, const int* n, int howmany, fftwf_complex* in, const int*, int istride,
                                   int idist, float* out, const int*, int ostride, int odist, unsigned) {
    if (rank != 2 || istride != 1 || ostride != 1) std::abort();
    return new fftwf_plan_s{C2R, n[0], n[1], FFTW_BACKWARD, howmany, idist, odist, nullptr, in, nullptr, out};
}

void fftwf_execute_dft(const fftwf_plan p, fftwf_complex* in, fftwf_complex* out) {
    const int n0 = p->n0, n1 = p->n1;
    std::vector<cd> a((size_t)n0 * n1);
    for (size_t i = 0; i < a.size(); ++i) a[i] = cd(in[i][0], in[i][1]);
    dft2(a, n0, n1, p->sign);
    for (size_t i = 0; i < a.size(); ++i) {
        out[i][0] = (float)a[i].real();
        out[i][1] = (float)a[i].imag();
    }
}

void fftwf_execute(const fftwf_plan p) {
    const int n0 = p->n0, n1 = p->n1, h = n1 / 2 + 1;
    if (p->kind == C2C) {
        fftwf_execute_dft(p, p->cin, p->cout);
        return;
    }
    for (int b = 0; b < p->howmany; ++b) {
        if (p->kind == R2C) {
            const float* x = p->rin + (size_t)b * p->idist;
            fftwf_complex* y = p->cout + (size_t)b * p->odist;
            std::vector<cd> a((size_t)n0 * n1);
            for (size_t i = 0; i < a.size(); ++i) a[i] = cd(x[i], 0.0);
            dft2(a, n0, n1, FFTW_FORWARD);
            for (int i = 0; i < n0; ++i)
                for (int j = 0; j < h; ++j) {
                    y[(size_t)i * h + j][0] = (float)a[(size_t)i * n1 + j].real();
                    y[(size_t)i * h + j][1] = (float)a[(size_t)i * n1 + j].imag();
                }
        } else {
            // inverse along the first dimension over the stored half, then a real inverse
            // along the last: the imaginary parts at frequency 0 (and n1 / 2 for even n1),
            // which a Hermitian row holds as zero, do not enter
            const fftwf_complex* x = p->cin + (size_t)b * p->idist;
            float* y = p->rout + (size_t)b * p->odist;
            std::vector<cd> a((size_t)n0 * h);
            for (size_t i = 0; i < a.size(); ++i) a[i] = cd(x[i][0], x[i][1]);
            dft2(a, n0, h, FFTW_BACKWARD, false, true);
            std::vector<cd> row(n1);
            for (int i = 0; i < n0; ++i) {
                for (int j = 0; j < h; ++j) row[j] = a[(size_t)i * h + j];
                row[0] = cd(row[0].real(), 0.0);
                if (n1 % 2 == 0) row[n1 / 2] = cd(row[n1 / 2].real(), 0.0);
                for (int j = h; j < n1; ++j) row[j] = std::conj(row[n1 - j]);
                dft1(row, FFTW_BACKWARD);
                for (int j = 0; j < n1; ++j) y[(size_t)i * n1 + j] = (float)row[j].real();
            }
        }
    }
}

}  // extern "C"
