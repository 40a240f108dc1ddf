// BandPassRecorder: the integrated spectrum and its polynomial model, the
// bandpass the RFI clipper subtracts.
//
// Follows lib/src/BandPassRecorder.cpp:22-190 as it is evidently meant to
// work: Stokes-I spectra (polarisation 0) are summed per channel until
// requiredSamples spectra have been added; the mean spectrum is fitted by a
// least-squares polynomial in frequency (BinMap from startFrequency to
// endFrequency, coefficients of f^0 .. f^(n-1)); channels more than 2 RMS
// of the residuals above the fit are replaced by the fit and the fit is
// repeated until none is; the bandpass RMS is that of the cleaned mean
// spectrum across channels.  The reference's own code cannot run (its
// LAPACK call takes the character 'N' as a pointer (:18), the right-hand
// side holds ncoeffs of nBins values (:53, :155), the matrix is row-major
// under a column-major leading dimension (:60), and the trim loop never
// clears its count (:106-129)), so this is a restatement of the intent, not
// of those lines.
//
// The sum over time is the only heavy part (every filterbank byte read
// once): each CTA owns 256 channels of a 256-spectrum segment and sums it in
// FP32 in time order; segment partials are added in FP64, in segment order,
// into the running sums.  The fit (a few coefficients) is FP64 Householder
// QR on the host.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "pv_internal.cuh"

namespace {

constexpr int kSeg = 256;  // spectra per partial sum

__global__ void __launch_bounds__(256)
spectrum_partial_kernel(const float* __restrict__ in, int nt, int npol, int nchan, int nbins,
                        float* __restrict__ part) {
    const int bin = blockIdx.x * blockDim.x + threadIdx.x;
    const int seg = blockIdx.y;
    if (bin >= nbins) return;
    const int s = bin / nchan, c = bin - s * nchan;
    const long long stride = (long long)(nbins / nchan) * npol * nchan;  // one spectrum
    const long long base = ((long long)s * npol) * nchan + c;           // polarisation 0
    const int t0 = seg * kSeg, t1 = min(nt, t0 + kSeg);
    float acc = 0.0f;
#pragma unroll 8
    for (int t = t0; t < t1; ++t) acc = __fadd_rn(acc, __ldg(in + base + (long long)t * stride));
    part[(long long)seg * nbins + bin] = acc;
}

__global__ void __launch_bounds__(256)
spectrum_accumulate_kernel(const float* __restrict__ part, int nseg, int nbins, double* __restrict__ acc) {
    const int bin = blockIdx.x * blockDim.x + threadIdx.x;
    if (bin >= nbins) return;
    double a = acc[bin];
    for (int k = 0; k < nseg; ++k) a = __dadd_rn(a, (double)part[(long long)k * nbins + bin]);
    acc[bin] = a;
}

// Least squares min |V x - y| by Householder QR; V is n x m, column-major.
bool lstsq(std::vector<double> V, std::vector<double> y, int n, int m, std::vector<double>& x) {
    for (int k = 0; k < m; ++k) {
        double norm = 0.0;
        for (int i = k; i < n; ++i) norm += V[(size_t)k * n + i] * V[(size_t)k * n + i];
        norm = std::sqrt(norm);
        if (norm == 0.0) return false;
        const double a = V[(size_t)k * n + k] > 0 ? -norm : norm;
        std::vector<double> v(V.begin() + (size_t)k * n + k, V.begin() + (size_t)k * n + n);
        v[0] -= a;
        double vv = 0.0;
        for (double e : v) vv += e * e;
        if (vv == 0.0) continue;
        for (int j = k; j < m; ++j) {
            double d = 0.0;
            for (int i = k; i < n; ++i) d += v[i - k] * V[(size_t)j * n + i];
            const double f = 2.0 * d / vv;
            for (int i = k; i < n; ++i) V[(size_t)j * n + i] -= f * v[i - k];
        }
        double d = 0.0;
        for (int i = k; i < n; ++i) d += v[i - k] * y[i];
        const double f = 2.0 * d / vv;
        for (int i = k; i < n; ++i) y[i] -= f * v[i - k];
    }
    x.assign(m, 0.0);
    for (int k = m - 1; k >= 0; --k) {
        double s = y[k];
        for (int j = k + 1; j < m; ++j) s -= V[(size_t)j * n + k] * x[j];
        const double r = V[(size_t)k * n + k];
        if (r == 0.0) return false;
        x[k] = s / r;
    }
    return true;
}

}  // namespace

struct pv_bandpass_recorder {
    long long required = 0, total = 0;
    int ncoeffs = 3, nbins = 0;
    float start = 0.0f, end = 0.0f;
    double* d_acc = nullptr;
    float* d_part = nullptr;
    long long part_cap = 0;
    bool ready = false;
    std::vector<float> coeffs;
    float rms = 0.0f;
    int trimmed = 0;
};

extern "C" int pv_bandpass_recorder_create(pv_bandpass_recorder** out, long long required_samples, int ncoeffs,
                                           float start_freq, float end_freq) {
    if (!out || ncoeffs < 1 || ncoeffs > 16 || required_samples < 0) {
        pv::set_error("BandPassRecorder: invalid arguments");
        return PV_ERR_ARG;
    }
    if (!(end_freq != start_freq)) {
        pv::set_error("BandPassRecorder: the band's start and end frequencies are equal");
        return PV_ERR_CONFIG;
    }
    auto* r = new pv_bandpass_recorder;
    r->required = required_samples;
    r->ncoeffs = ncoeffs;
    r->start = start_freq;
    r->end = end_freq;
    *out = r;
    return PV_OK;
}

extern "C" void pv_bandpass_recorder_destroy(pv_bandpass_recorder* r) {
    if (!r) return;
    cudaFree(r->d_acc);
    cudaFree(r->d_part);
    delete r;
}

namespace {

int fit(pv_bandpass_recorder* r, const std::vector<double>& sum) {
    const int n = r->nbins, m = r->ncoeffs;
    if (n < m) {
        pv::set_error("BandPassRecorder: %d channels cannot fit %d coefficients", n, m);
        return PV_ERR_ARG;
    }
    // BinMap(nBins) from start to end: width (end - start) / nBins, bin i at start + i * width
    const double width = ((double)r->end - (double)r->start) / n;
    std::vector<double> f(n), y(n), V((size_t)n * m);
    for (int i = 0; i < n; ++i) {
        f[i] = (double)(float)((double)r->start + width * i);
        y[i] = sum[i] / (double)r->total;
        double p = 1.0;
        for (int k = 0; k < m; ++k, p *= f[i]) V[(size_t)k * n + i] = p;
    }
    std::vector<double> x;
    auto eval = [&](double v) {
        double tot = 0.0, p = 1.0;
        for (int k = 0; k < m; ++k, p *= v) tot += x[k] * p;
        return tot;
    };
    r->trimmed = 0;
    for (int iter = 0; iter < 1000; ++iter) {
        if (!lstsq(V, y, n, m, x)) {
            pv::set_error("BandPassRecorder: the frequency matrix does not have full rank");
            return PV_ERR_ARG;
        }
        double rs = 0.0, rss = 0.0;
        for (int i = 0; i < n; ++i) {
            const double res = y[i] - eval(f[i]);
            rs += res;
            rss += res * res;
        }
        const double margin = 2.0 * std::sqrt(std::max(0.0, rss / n - (rs / n) * (rs / n)));
        int cut = 0;
        for (int i = 0; i < n; ++i)
            if (y[i] - eval(f[i]) > margin) {
                y[i] = eval(f[i]);
                ++cut;
            }
        r->trimmed += cut;
        if (cut == 0) break;
    }
    double s = 0.0, ss = 0.0;
    for (int i = 0; i < n; ++i) {
        s += y[i];
        ss += y[i] * y[i];
    }
    r->rms = (float)std::sqrt(std::max(0.0, ss / n - (s / n) * (s / n)));
    r->coeffs.assign(x.begin(), x.end());
    r->ready = true;
    return PV_OK;
}

}  // namespace

extern "C" int pv_bandpass_recorder_add(pv_bandpass_recorder* r, const float* d_stokes, int nt, int nsub, int npol,
                                        int nchan, void* stream) {
    if (!r || !d_stokes || nt < 0 || nsub <= 0 || npol <= 0 || nchan <= 0) {
        pv::set_error("pv_bandpass_recorder_add: invalid arguments");
        return PV_ERR_ARG;
    }
    cudaStream_t s = pv::as_stream(stream);
    const int nbins = nsub * nchan;
    if (nbins != r->nbins || r->total == 0 || r->ready) {  // a new integration (BandPassRecorder.cpp:85)
        cudaFree(r->d_acc);
        r->d_acc = nullptr;
        PV_CUDA(cudaMalloc(&r->d_acc, sizeof(double) * nbins), "allocate bandpass sums");
        PV_CUDA(cudaMemsetAsync(r->d_acc, 0, sizeof(double) * nbins, s), "clear bandpass sums");
        r->nbins = nbins;
        r->total = 0;
        r->ready = false;
    }
    if (nt > 0) {
        const int nseg = (nt + kSeg - 1) / kSeg;
        if (nseg > 65535) {
            pv::set_error("pv_bandpass_recorder_add: more than %d spectra in one call", 65535 * kSeg);
            return PV_ERR_ARG;
        }
        if ((long long)nseg * nbins > r->part_cap) {
            cudaFree(r->d_part);
            r->d_part = nullptr;
            r->part_cap = (long long)nseg * nbins;
            PV_CUDA(cudaMalloc(&r->d_part, sizeof(float) * r->part_cap), "allocate bandpass partials");
        }
        const dim3 grid((unsigned)pv::ceil_div(nbins, 256), (unsigned)nseg);
        spectrum_partial_kernel<<<grid, 256, 0, s>>>(d_stokes, nt, npol, nchan, nbins, r->d_part);
        PV_TRY(pv::check_launch("spectrum_partial_kernel"));
        spectrum_accumulate_kernel<<<pv::ceil_div(nbins, 256), 256, 0, s>>>(r->d_part, nseg, nbins, r->d_acc);
        PV_TRY(pv::check_launch("spectrum_accumulate_kernel"));
        r->total += nt;
    }
    if (r->total < r->required || r->total == 0) return 0;  // collect more data
    std::vector<double> sum(nbins);
    PV_CUDA(cudaMemcpyAsync(sum.data(), r->d_acc, sizeof(double) * nbins, cudaMemcpyDeviceToHost, s),
            "read bandpass sums");
    PV_CUDA(cudaStreamSynchronize(s), "read bandpass sums");
    PV_TRY(fit(r, sum));
    return 1;
}

extern "C" int pv_bandpass_recorder_result(const pv_bandpass_recorder* r, float* h_coeffs, float* h_rms,
                                           int* h_trimmed, char* h_bp_text, long long cap, long long* h_len) {
    if (!r || !r->ready) {
        pv::set_error("BandPassRecorder: no fit yet");
        return PV_ERR_ARG;
    }
    for (int k = 0; k < r->ncoeffs; ++k)
        if (h_coeffs) h_coeffs[k] = (float)r->coeffs[k];
    if (h_rms) *h_rms = r->rms;
    if (h_trimmed) *h_trimmed = r->trimmed;
    if (!h_len) return PV_OK;
    // BandPassAdapter format (lib/src/BandPassAdapter.cpp:30-108): nChan, start, end, width, rms,
    // then the polynomial, constant term first (the adapter also takes it as the median)
    std::string t = "# BandPassRecorder\n";
    char line[64];
    const double width = ((double)r->end - (double)r->start) / r->nbins;
    std::snprintf(line, sizeof line, "%d\n%.9g\n%.9g\n%.17g\n%.9g\n", r->nbins, (double)r->start, (double)r->end,
                  width, (double)r->rms);
    t += line;
    for (int k = 0; k < r->ncoeffs; ++k) {
        std::snprintf(line, sizeof line, "%.9g\n", (double)(float)r->coeffs[k]);
        t += line;
    }
    *h_len = (long long)t.size();
    if (h_bp_text && (long long)t.size() <= cap) std::memcpy(h_bp_text, t.data(), t.size());
    if (h_bp_text && (long long)t.size() > cap) {
        pv::set_error("pv_bandpass_recorder_result: %lld bytes needed", (long long)t.size());
        return PV_ERR_ARG;
    }
    return PV_OK;
}
