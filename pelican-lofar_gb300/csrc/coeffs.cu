// A2: polyphase filter coefficients (PolyphaseCoefficients::genereateFilter,
// lib/src/PolyphaseCoefficients.cpp:77-364), host-side set-up.
//
// The design is Octave's fir2 with grid_n = nextpow2(order+1) and a ramp of
// ramp_n/grid_n, which integer division makes 0: the ideal response is 1
// below w = 1/nChannels and 0 above.  The reference inverts it with a
// single-precision FFTW backward transform of length 4*grid_n; here the
// needed outputs are summed directly in double and rounded to float, which
// is the correctly rounded value of that transform.  The response is then
// windowed, normalised by its centre tap, scaled by 1/nChannels and given
// the alternating channel sign (-1)^c.
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "pv_common.cuh"

namespace pv {

namespace {

double bessel_i0_poly(double x) {
    // Polynomial approximation of I0 (Abramowitz & Stegun 9.8.1/9.8.2), the
    // one PolyphaseCoefficients.cpp:77-103 uses.
    const double ax = std::fabs(x);
    if (ax < 3.75) {
        const double y = (x / 3.75) * (x / 3.75);
        return 1.0 + y * (3.5156229 + y * (3.0899424 + y * (1.2067492 + y * (0.2659732 +
               y * (3.60768e-2 + y * 4.5813e-3)))));
    }
    const double y = 3.75 / ax;
    return (std::exp(ax) / std::sqrt(ax)) *
           (0.39894228 + y * (1.328592e-2 + y * (2.25319e-3 + y * (-1.57565e-3 + y * (9.16281e-3 +
            y * (-2.057706e-2 + y * (2.635537e-2 + y * (-1.647633e-2 + y * 3.92377e-3))))))));
}

std::vector<double> make_window(unsigned n, int type) {
    std::vector<double> w(n, 1.0);
    if (n == 1) return w;
    const unsigned m = n - 1;
    switch (type) {
        case PV_WINDOW_HAMMING:  // symmetric, PolyphaseCoefficients.cpp:139-149
            for (unsigned i = 0; i < n; ++i) w[i] = 0.54 - 0.46 * std::cos((2.0 * M_PI * i) / m);
            break;
        case PV_WINDOW_BLACKMAN:  // i/m is an integer division there (:160): k is 0 or 1
            for (unsigned i = 0; i < n; ++i) {
                const double k = (double)(i / m);
                w[i] = 0.42 - 0.5 * std::cos(2.0 * M_PI * k) + 0.08 * std::cos(4.0 * M_PI * k);
            }
            break;
        case PV_WINDOW_GAUSSIAN: {  // alpha 3.5, :130-136
            const double a = 3.5;
            unsigned idx = 0;
            for (int i = -(int)(n - 1); i <= (int)(n - 1); i += 2) {
                const double x = a / (int)n * i;
                w[idx++] = std::exp(-0.5 * (x * x));
            }
            break;
        }
        default: {  // Kaiser beta 9.0695, :114-127
            const double beta = 9.0695;
            for (unsigned i = 0; i < n; ++i) {
                const double k = 2.0 * beta / (int)m * std::sqrt(double((int)i * ((int)m - (int)i)));
                w[i] = bessel_i0_poly(k) / bessel_i0_poly(beta);
            }
        }
    }
    return w;
}

}  // namespace

int fir_coefficients(int ntaps, int nchan, int window, std::vector<double>& out) {
    const unsigned total = (unsigned)ntaps * (unsigned)nchan;
    if (ntaps <= 0 || nchan <= 0 || total < 2) {
        set_error("PolyphaseCoefficients: need at least two coefficients");
        return PV_ERR_ARG;
    }
    const unsigned order = total - 1;
    unsigned grid_n = 1;
    while (grid_n < order + 1) grid_n *= 2;
    const double w = 1.0 / nchan;
    // Ideal response sampled at grid_n+1 points of [0,1]: 1 below w, 0 from w.
    std::vector<double> grid(grid_n + 1);
    for (unsigned i = 0; i <= grid_n; ++i) {
        const double x = (double)i / grid_n;
        grid[i] = x < w ? 1.0 : 0.0;
    }
    // Real even input of the length-L inverse transform (float values), and
    // the real part of the outputs the design keeps.
    const unsigned L = 4 * grid_n;
    std::vector<double> in(L, 0.0);
    for (unsigned i = 0; i <= grid_n; ++i) in[i] = (float)grid[i];
    for (unsigned i = 1; i < grid_n; ++i) in[3 * grid_n + i] = (float)grid[grid_n - i];
    auto re_out = [&](unsigned k) {
        double s = 0.0;
        for (unsigned j = 0; j < L; ++j) {
            if (in[j] == 0.0) continue;
            s += in[j] * std::cos(2.0 * M_PI * (double)((unsigned long long)j * k % L) / L);
        }
        return (double)(float)s;
    };
    std::vector<double> h(total);
    unsigned idx = 0;
    for (unsigned i = L - order; i < L; i += 2) h[idx++] = re_out(i);
    for (unsigned i = 1; i <= order; i += 2) h[idx++] = re_out(i);
    const std::vector<double> win = make_window(total, window);
    for (unsigned i = 0; i < total; ++i) h[i] *= win[i];
    const double centre = h[order / 2];
    for (unsigned i = 0; i < total; ++i) h[i] /= centre;
    out.assign(total, 0.0);
    for (int t = 0; t < ntaps; ++t)
        for (int c = 0; c < nchan; ++c) {
            const unsigned i = t * nchan + c;
            out[i] = (c % 2 == 0) ? h[i] / nchan : -h[i] / nchan;
        }
    return PV_OK;
}

}  // namespace pv

extern "C" int pv_fir_coefficients(int ntaps, int nchan, int window, double* h_coeffs) {
    if (!h_coeffs) {
        pv::set_error("pv_fir_coefficients: null output");
        return PV_ERR_ARG;
    }
    std::vector<double> c;
    PV_TRY(pv::fir_coefficients(ntaps, nchan, window, c));
    std::memcpy(h_coeffs, c.data(), sizeof(double) * c.size());
    return PV_OK;
}

extern "C" int pv_window_from_name(const char* name) {
    if (!name) return -1;
    std::string s(name);
    for (auto& ch : s) ch = (char)std::tolower((unsigned char)ch);
    if (s == "kaiser") return PV_WINDOW_KAISER;
    if (s == "gaussian") return PV_WINDOW_GAUSSIAN;
    if (s == "blackman") return PV_WINDOW_BLACKMAN;
    if (s == "hamming") return PV_WINDOW_HAMMING;
    pv::set_error("PPFChanneliser: Unknown coefficient window type '%s'.", name);
    return -1;
}
