/*
 * pv.h — C ABI of the GB300 (sm_103a) beam-processing library (libpv.so).
 *
 * The library replaces the hot path of pelican-lofar:
 *   PPFChanneliser -> StokesGenerator -> StokesIntegrator -> RFI_Clipper
 *   -> DedispersionModule (DedispersionBuffer + cache_dedisperse_loop)
 *   -> DedispersionAnalyser.
 * Reference citations are relative to pelican-lofar's src/ directory.
 *
 * Conventions
 *  - Every function returns PV_OK (0) or a negative PV_ERR_* code and never
 *    throws.  pv_last_error() returns the calling thread's last message.
 *  - "d_" pointers are device pointers, "h_" pointers host pointers.
 *  - stream is a cudaStream_t passed as void* (NULL = the legacy default
 *    stream).  Device-pointer calls are asynchronous on that stream.
 *  - Layouts are the reference's data-set layouts (see each declaration).
 */
#ifndef PV_H
#define PV_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PV_OK 0
#define PV_ERR_ARG -1      /* invalid argument / shape */
#define PV_ERR_CUDA -2     /* CUDA runtime error */
#define PV_ERR_CONFIG -3   /* configuration error (reference: throw QString) */
#define PV_ERR_NOMEM -4    /* allocation failed */
#define PV_ERR_STATE -5    /* call out of sequence */
#define PV_ERR_TIMEOUT -6  /* a bounded device wait gave up */
#define PV_ERR_NODEV -7    /* no CUDA device */

const char* pv_last_error(void);
int pv_version(void);
/* Number of kernels this library launched since load (all entry points). */
long long pv_kernel_launches(void);

/* ------------------------------------------------------------------------
 * A7 delay table — DedispersionModule::resize (lib/src/DedispersionModule.cpp:109-190)
 * ---------------------------------------------------------------------- */

/* dmshift[c] = (float)(4148.741601*(1/f_c^2 - 1/f_1^2)), f_c = fch1 + foff*c.
 * Bands with foff >= 0 ("inverted", DedispersionModule.cpp:60) are handled
 * with the highest frequency first so every delay is >= 0; *inverted is set
 * and the caller fills the buffer in reversed channel order
 * (DedispersionBuffer.cpp:131-156).  Host function. */
int pv_dm_shifts(double fch1, double foff, int nchan, float* h_dmshift, int* inverted);

/* maxshift and remainingSamples exactly as DedispersionModule::resize
 * (DedispersionModule.cpp:159,162).  Host function. */
int pv_maxshift(float dm_low, float dm_step, int tdms, const float* h_dmshift, int nchan,
                double tsamp, int buffer_samples, int* maxshift, int* remaining);

/* K0: integer delay table shifts[d*nchan + c] =
 * trunc_f32(dmshift[c] * fmaf(d, step_over_tsamp, start_over_tsamp))
 * (the per-thread shift of DedispersionKernel.cu:29,36), on the device. */
int pv_delay_table(int* d_shifts, const float* d_dmshift, int nchan, int tdms,
                   float start_over_tsamp, float step_over_tsamp, void* stream);

/* ------------------------------------------------------------------------
 * A9 dedispersion — replaces cacheDedisperseLoop (lib/DedispersionKernel.cu:53-86)
 * ---------------------------------------------------------------------- */

/* Same arguments and meaning as the reference's
 *   cacheDedisperseLoop(float* outbuff, long outbufSize, float* buff,
 *                       float mstartdm, float mdmstep, int tdms, int numSamples,
 *                       const float* dmShift, int maxshift, int i_nchans)
 * buff is [nchans][numSamples] (DedispersionBuffer layout), outbuff is
 * [tdms][numSamples - maxshift] (DedispersionSpectra layout); mstartdm and
 * mdmstep are dmLow/tsamp and dmStep/tsamp.  Unlike the reference launch
 * every trial 0..tdms-1 is computed for any tdms.  Asynchronous on stream. */
int pv_dedisperse(float* d_out, long long out_bytes, const float* d_in, float start_over_tsamp,
                  float step_over_tsamp, int tdms, int num_samples, const float* d_dmshift,
                  int maxshift, int nchans, void* stream);

/* General form: input rows of row_stride floats holding row_len valid
 * samples; nout outputs per trial written with out_stride.  Samples at or
 * beyond row_len read as 0. */
int pv_dedisperse_ex(float* d_out, long long out_stride, const float* d_in,
                     long long row_stride, long long row_len, int nchans, int nout, int tdms,
                     const float* d_dmshift, float start_over_tsamp, float step_over_tsamp,
                     void* stream);

/* A dedispersion plan: the delay constants (host and device copies) and the
 * tile choice for one channel set and trial grid, so that repeated launches
 * need no host synchronisation.  h_dmshift is copied. */
typedef struct pv_dedisp_plan pv_dedisp_plan;
int pv_dedisp_plan_create(pv_dedisp_plan** plan, const float* h_dmshift, int nchans, int tdms,
                          float start_over_tsamp, float step_over_tsamp);
void pv_dedisp_plan_destroy(pv_dedisp_plan* plan);
/* Largest integer delay of the plan (samples). */
int pv_dedisp_plan_max_shift(const pv_dedisp_plan* plan);
/* Dedisperses nout samples.  Linear mode (ring_len == 0): rows of row_stride
 * floats, samples at or beyond row_len read as 0 (row_len == row_stride reads
 * on into the next row, as the reference's contiguous buffer does).  Ring
 * mode (ring_len > 0): each row is a ring of ring_len samples and output
 * sample t reads physical column (t_base + t + shift) mod ring_len. */
int pv_dedisp_plan_run(const pv_dedisp_plan* plan, float* d_out, long long out_stride,
                       const float* d_in, long long row_stride, long long row_len,
                       long long ring_len, long long t_base, int nout, void* stream);

/* A8 DedispersionBuffer::addSamples (lib/src/DedispersionBuffer.cpp:98-180):
 * writes nt Stokes samples [t][nsub][npol][nchan] (pol 0) into the rows of a
 * per-channel ring at logical position pos (column (pos+t) mod ring_len; with
 * ring_len == 0 the rows are linear).  Row r takes bin r, or bin
 * nsub*nchan-1-r when inverted (DedispersionBuffer.cpp:131-156). */
int pv_ring_write(float* d_ring, long long row_stride, long long ring_len, long long pos,
                  const float* d_stokes, int nt, int nsub, int npol, int nchan, int inverted,
                  void* stream);

/* ------------------------------------------------------------------------
 * A11 analyser — DedispersionAnalyser::analyse (lib/src/DedispersionAnalyser.cpp:30-203)
 * ---------------------------------------------------------------------- */

typedef struct {
    int32_t dm;       /* DM trial index */
    int32_t t;        /* sample index in the DedispersionSpectra */
    float bin_factor; /* matched-filter width 2^n (DedispersionEvent mfBinning) */
    float value;      /* boxcar sum (DedispersionEvent mfValue) */
} pv_event;

/* Thresholds for levels 0..bin_pow2: level 0 = threshold*rms (float), level
 * n = threshold*rms*sqrt(2^n) (DedispersionAnalyser.cpp:112,121).  Host. */
int pv_analyser_thresholds(float threshold, float rms, int bin_pow2, float* h_thr);

/* Events of data [tdms][nsamp] (row stride ld) in the reference order: the
 * dummy (0,0,1,0) first, then by DM, 2^bin_pow2 block, width, position.
 * d_events receives at most cap events; *h_count (host) receives the total
 * including the dummy.  rms is the DedispersionDataAnalysis RMS
 * (sqrt(nChannels*nSubbands), DedispersionAnalyser.cpp:38).  Synchronises
 * the stream to read the count back. */
int pv_analyse(const float* d_data, long long ld, int tdms, int nsamp, float threshold,
               float rms, int bin_pow2, pv_event* d_events, long long cap,
               long long* h_count, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* PV_H */
