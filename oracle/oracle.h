/*
 * CPU oracle for the pelican-lofar beam-processing hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: the parity tests,
 * the smoke check and the CPU-baseline leg of the benchmark load it.  The
 * product library never links, loads or calls it.
 *
 * Every function restates one step of the reference (pelican-lofar, paths
 * relative to its src/ directory) from the behaviour of its source; the
 * citation is given beside each declaration.  Floating-point expressions
 * follow the reference's evaluation order and types (the reference builds
 * as C++98 with x86-64 SSE arithmetic: no fused multiply-add, float
 * std::pow(float,int), double ::sqrt).  This file is compiled with
 * -ffp-contract=off so that the same holds on aarch64.
 */
#ifndef PV_ORACLE_H
#define PV_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- A7: delay table (lib/src/DedispersionModule.cpp:151-162) ----------- */

/* Per-channel delay constants dmshift[c] = (float)(4148.741601*(1/f_c^2 - 1/f_1^2))
 * for f_c = fch1 + foff*c.  Inverted bands (foff >= 0) are re-expressed in
 * descending order (fch1' = fch1 + foff*(n-1), foff' = -foff) so that every
 * delay is >= 0.  Returns 1 if the band was inverted, else 0. */
int or_dm_shifts(double fch1, double foff, int nchan, float* dmshift);

/* maxshift and remainingSamples of DedispersionModule::resize
 * (DedispersionModule.cpp:159,162) for the descending table. */
void or_maxshift(float dm_low, float dm_step, int tdms, const float* dmshift,
                 int nchan, double tsamp, int buffer_samples,
                 int* maxshift, int* remaining);

/* Integer shift of channel c at trial d as the reference kernel computes it
 * (lib/DedispersionKernel.cu:29,36): trunc_f32(dmshift[c] * fmaf(d, step, start)).
 * mode 0 = that FP32 form; mode 1 = FP64 form trunc(dmshift64[c]*(dmLow+d*dmStep)/tsamp)
 * with dmshift64 computed in double (fch1/foff needed for mode 1). */
void or_shift_table(const float* dmshift, int nchan, int tdms,
                    float start_over_tsamp, float step_over_tsamp, int* shifts);
void or_shift_table_f64(double fch1, double foff, int nchan, int tdms,
                        double dm_low, double dm_step, double tsamp, int* shifts);

/* ---- A9: brute-force dedispersion (lib/DedispersionKernel.cu:15-50) ------ */

/* out[d*nout + t] = sum_{c=0..nchan-1} buf[c*ld + t + shift(c,d)], summed in
 * channel order in FP32 (the reference kernel's per-thread order), every trial
 * 0..tdms-1 computed.  nthreads<=0 uses all OpenMP threads. */
void or_dedisperse(const float* buf, int nchan, long long ld, int nout, int tdms,
                   const float* dmshift, float start_over_tsamp,
                   float step_over_tsamp, float* out, int nthreads);
/* Same sum in FP64 (error reference); out is double. */
void or_dedisperse_f64(const float* buf, int nchan, long long ld, int nout, int tdms,
                       const float* dmshift, float start_over_tsamp,
                       float step_over_tsamp, double* out, int nthreads);

/* ---- A11: analyser (lib/src/DedispersionAnalyser.cpp:30-203) ------------ */

typedef struct {
    int32_t dm;        /* DM trial index */
    int32_t t;         /* sample index within the DedispersionSpectra */
    float bin_factor;  /* boxcar width 2^n */
    float value;       /* boxcar sum */
} or_event;

/* Detection thresholds for levels n = 0..bin_pow2 (level 0 is thr*rms in
 * float, level n multiplies by ::sqrt(double(2^n))). */
void or_thresholds(float thr, float rms, int bin_pow2, float* out);
/* Appends the dummy event (0,0,1,0) and every event in the reference order.
 * Returns the number of events (including the dummy); writes at most cap. */
long long or_analyse(const float* data, int tdms, int nsamp, float thr, float rms,
                     int bin_pow2, or_event* events, long long cap);

/* ---- A2: polyphase coefficients (lib/src/PolyphaseCoefficients.cpp:77-364) */

/* window: 0 hamming, 1 blackman, 2 gaussian, 3 kaiser.  coeffs[t*nchan+c]. */
int or_fir_coefficients(int ntaps, int nchan, int window, double* coeffs);

/* ---- A3: PPF channeliser (lib/src/PPFChanneliser.cpp:81-290) ------------ */

typedef struct or_ppf or_ppf;
or_ppf* or_ppf_create(int nchan, int ntaps, const float* coeffs /* [ntaps][nchan] */);
void or_ppf_destroy(or_ppf*);
/* in: complex float [sub][pol][block][nchan] (TimeSeriesDataSetC32 layout,
 * nTimesPerBlock = nchan).  out: complex float [block][sub][pol][nchan]
 * (SpectrumDataSetC32 layout).  The FFT is computed in FP64 from the float
 * filter output and rounded to float (FFTW itself is absent). */
int or_ppf_run(or_ppf*, const float* in, int nsub, int npol, int nblocks, float* out);

/* ---- A4: Stokes (lib/src/StokesGenerator.cpp:40-108) -------------------- */
/* spectra: complex [t][sub][2][nchan]; stokes: float [t][sub][nstokes][nchan] */
void or_stokes(const float* spectra, int nt, int nsub, int nchan, int nstokes, float* stokes);

/* ---- A5: integrator (lib/src/StokesIntegrator.cpp:32-119) -------------- */
/* Returns the number of output samples; out [u][sub][npol][nchan/bin]. */
int or_integrate(const float* in, int nt, int nsub, int npol, int nchan,
                 int window, int bin_chans, float* out);

/* ---- A6: bandpass + RFI clipper (lib/src/RFI_Clipper.cpp:22-573,
 *          BandPass.cpp, BandPassAdapter.cpp:30-108, BinMap.cpp) ---------- */

typedef struct or_rfi or_rfi;
/* bp_text: the .bp file contents.  mode 0 restates the reference's FP32
 * arithmetic with sequential channel sums.  mode 1 is the FP64 variant the
 * library implements: per-channel arithmetic in the reference's FP32 form,
 * channel sums as `parts` FP32 partials (partial p takes channels p, p+parts,
 * ...) reduced by an FP64 tree (or_sum_canonical), and the per-spectrum
 * statistics and running averages in double.  Returns NULL and fills err
 * (if given) on a parse error. */
or_rfi* or_rfi_create(const char* bp_text, float cr_factor, float sr_factor,
                      int max_history, int zero_dming, int use_mean_over_rms,
                      int band_matching, int mode, int parts, char* err, int errlen);
void or_rfi_destroy(or_rfi*);
/* In-place on I [t][sub][npol][nchan]; weights (same shape) are set to 1
 * where the reference writes them.  flags (optional, [t][nbins] uint8):
 * bit0 channel clipped, bit1 spectrum clipped. */
int or_rfi_run(or_rfi*, float* data, float* weights, int nt, int nsub, int npol,
               int nchan, uint8_t* flags);
/* or_rfi_run with another implementation's flags as a guide (hint
 * [t][nbins], the layout of `flags`).  Where this run's channel or spectrum
 * decision differs from the hint and its decision statistic lies within eps
 * of the threshold (channel: |(I - dataModel - bp) - margin| <= eps_chan *
 * rmsRunAve; spectrum: |(mean - meanRunAve) - tolerance| <= eps_spec *
 * bandpass rms / sqrt(nBins)), the hint's decision is taken; every other
 * difference is a mismatch, after which the hint is followed as well so the
 * two runs keep one state.  report12: [channel decisions, channel
 * differences within eps, channel mismatches, largest |statistic| of a
 * channel difference within eps, spectrum decisions, spectrum differences
 * within eps, spectrum mismatches, largest |statistic| of those, smallest
 * |statistic| of any channel decision, smallest |statistic| of any spectrum
 * rejection test, first spectrum with a difference (-1: none), 0]
 * (statistics in their eps units). */
int or_rfi_run_guided(or_rfi*, float* data, float* weights, int nt, int nsub, int npol, int nchan,
                      const uint8_t* hint, double eps_chan, double eps_spec, uint8_t* flags,
                      double* report12);
/* Scalar state after the last run: [meanRunAve, rmsRunAve, bp_mean, bp_rms,
 * params0, num, badSpectra, meanBufferSize, rmsBufferSize, remainingZeros]. */
void or_rfi_state(const or_rfi*, double* out10);
/* Current bandpass values for nbins channels (after reBin of the last run). */
int or_rfi_bandpass(const or_rfi*, float* out, int nbins);

/* Canonical FP64 reduction used by the FP64 RFI variant: 256 strided
 * sequential partials followed by a halving pairwise tree. */
double or_sum_canonical(const float* x, int n, int parts);

/* BandPass/BinMap checks against the reference's own unit tests. */
typedef struct or_bandpass or_bandpass;
or_bandpass* or_bandpass_create(int nbins, double start, double width,
                                const float* params, int nparams);
void or_bandpass_destroy(or_bandpass*);
void or_bandpass_set_rms(or_bandpass*, float);
void or_bandpass_set_median(or_bandpass*, float);
void or_bandpass_set_mean(or_bandpass*, float);
void or_bandpass_kill_band(or_bandpass*, float start, float end);
void or_bandpass_rebin(or_bandpass*, int nbins, double start, double width);
float or_bandpass_intensity(const or_bandpass*, float freq);
float or_bandpass_intensity_of_bin(const or_bandpass*, int i);
float or_bandpass_median(const or_bandpass*);
float or_bandpass_rms(const or_bandpass*);
float or_bandpass_mean(const or_bandpass*);
int or_binmap_index(double start, double width, double value);

/* ---- A8/A10: DedispersionBuffer + DedispersionModule streaming ---------- */

typedef struct or_ddmod or_ddmod;
/* buffer_samples = 2^timeBinsPerBufferPow2 */
or_ddmod* or_ddmod_create(int buffer_samples, int tdms, float dm_low, float dm_step,
                          double fch1, double foff);
void or_ddmod_destroy(or_ddmod*);
/* Feed one Stokes blob [t][sub][npol][nchan] (pol 0 used).  Returns the
 * number of DedispersionSpectra completed by this call (retrieve with
 * or_ddmod_pop).  Returns -1 if maxshift does not fit the buffer. */
int or_ddmod_add(or_ddmod*, const float* stokes, int nt, int nsub, int npol,
                 int nchan, double tsamp);
/* Pops the oldest completed spectra.  Returns nout (samples per trial) and
 * writes tdms*nout floats into out (if cap allows) and the absolute first
 * sample index of the buffer. */
int or_ddmod_pop(or_ddmod*, float* out, long long cap, long long* first_sample);
void or_ddmod_params(const or_ddmod*, int* maxshift, int* remaining, int* nout,
                     int* nchan_total, int* inverted);

/* ---- Timing helper for the CPU baseline --------------------------------- */
int or_num_threads(void);

/* ---- F1 LOFAR UDP packets (AdapterTimeSeriesDataSet) --------------------- */
int or_udp_check(int fixed, int bits, int npackets, int spp, int nchan, int nsub, int npol,
                 long long chunk_bytes, long long* packet_bytes, int* nblocks);
/* out: complex float [nsub][npol][npackets*spp] */
int or_udp_unpack(const unsigned char* chunk, long long packet_bytes, int npackets, int bits,
                  int nsub, int npol, int spp, float* out);
void or_udp_time(const unsigned char* header, int clock_mhz, double* timestamp,
                 double* block_rate);

/* ---- F2 SigprocStokesWriter data block ----------------------------------- */
long long or_sigproc_pack(const float* stokes, int nt, int nsub, int npol, int nchan, int npw,
                          int nbits, float cmin, float cmax, unsigned char* out);

#ifdef __cplusplus
}
#endif
#endif
