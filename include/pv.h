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
/* Limit (ns) of each bounded device-side wait of the pipelined dedispersion
 * kernels launched from now on (ns <= 0: the default, 0.5 s).  A wait that
 * runs out makes the kernel record PV_ERR_TIMEOUT, wait for its own copies
 * in flight (up to 0.5 s) and return; the launch's other CTAs stop, and the
 * status reaches the caller through pv_dedisp_plan_status, pv_beam_events or
 * pv_batch_events.  A CUDA graph keeps the limit it was captured with.
 * Returns the previous limit.  No counterpart in the reference, whose
 * GPU_Job reports failures as GPU_Job::Failed (lib/src/GPU_Manager.cpp). */
long long pv_set_wait_limit(long long ns);
/* Failure-path test hook: the next n pipelined dedispersion launches (single
 * beam, plan or pv_dedisperse on ring rows) withhold the copies of their
 * first channel stage in every CTA, so the consumers' wait on that stage
 * can only end at the wait limit.  Nothing faults or hangs: the kernel
 * records PV_ERR_TIMEOUT and returns, as for a copy that never lands.
 * Returns the previous count. */
int pv_stall_next_launches(int n);
/* cudaMemcpyAsync with cudaMemcpyDefault (host or device pointers). */
int pv_device_copy(void* dst, const void* src, long long bytes, void* stream);
/* Page-locked host memory for input staging (cudaHostAlloc, portable).
 * write_combined = 1 makes it write-combined (uncached on the host).  On
 * GB300 (Grace host) the copy engine read write-combined staging at 91 GB/s
 * and ordinary page-locked staging at up to 211 GB/s, but at 60-165 GB/s
 * when it was allocated before the engine's device memory: stage with 0,
 * allocated after pv_batch_create. */
int pv_host_alloc(void** h_ptr, long long bytes, int write_combined);
void pv_host_free(void* h_ptr);
/* Device memory for callers without CUDA headers (the C++ module shim). */
int pv_device_alloc(void** d_ptr, long long bytes);
void pv_device_free(void* d_ptr);
/* Waits for the work issued on `stream`. */
int pv_synchronize(void* stream);

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
/* PV_OK, or PV_ERR_TIMEOUT if a pipelined launch's bounded wait gave up
 * (synchronous read of the plan's device status word). */
int pv_dedisp_plan_status(const pv_dedisp_plan* plan, int* h_status);
/* Clears a recorded PV_ERR_TIMEOUT so that the plan's next launch runs
 * (launches stop at their start while the status word holds an error). */
int pv_dedisp_plan_clear_status(pv_dedisp_plan* plan, void* stream);
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

/* A10 DedispersionModule::dedisperse with the reference's buffering
 * (lib/src/DedispersionModule.cpp:109-325): buffers of buffer_samples =
 * 2^timeBinsPerBufferPow2 samples, nout = buffer_samples - maxshift -
 * remainingSamples outputs per full buffer, the next buffer starting with the
 * previous one's last maxshift + remainingSamples samples.  Arguments follow
 * the XML keys dedispersionSamples, dedispersionMinimum, dedispersionStepSize,
 * frequencyChannel1@MHz, channelBandwidth@MHz. */
typedef struct pv_ddmod pv_ddmod;
int pv_ddmod_create(pv_ddmod** mod, int buffer_samples, int tdms, float dm_low, float dm_step,
                    double fch1, double foff);
void pv_ddmod_destroy(pv_ddmod* mod);
/* Adds one Stokes blob [nt][nsub][npol][nchan] (host or device pointer; pol
 * 0 is dedispersed) whose samples are tsamp seconds apart (the blob's
 * getBlockRate()).  *completed receives the number of buffers that became
 * full and were dedispersed (asynchronously on stream).  A maxshift larger
 * than the buffer is a PV_ERR_CONFIG with the reference's message. */
int pv_ddmod_add(pv_ddmod* mod, const float* stokes, int nt, int nsub, int npol, int nchan,
                 double tsamp, int* completed, void* stream);
/* Pops the oldest completed DedispersionSpectra: [tdms][nout] floats into out
 * (host or device, cap_floats >= tdms*nout; NULL discards it), *nout (0 when
 * none is ready) and the absolute index of its first input sample. */
int pv_ddmod_pop(pv_ddmod* mod, float* out, long long cap_floats, int* nout,
                 long long* first_sample, void* stream);
/* [maxshift, remainingSamples, nout, channels, inverted, completed buffers queued] */
int pv_ddmod_params(const pv_ddmod* mod, int* h_out6);

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

/* pv_analyse for callers that cannot allocate device memory.  This entry
 * point has no counterpart in the reference.  It exists for code that must
 * not call cudaMalloc once it runs: a real-time beam pipeline whose device
 * memory was reserved up front under a fixed HBM budget (an allocation there
 * would break the budget and stall the stream), or a host embedded in a
 * framework that owns the device allocator.
 *
 * Same arguments and results as pv_analyse.  Its scratch (per-block event
 * counts, offsets and scan workspace) is a fixed array in device memory
 * that every GPU loading the library keeps until the process exits.  It
 * holds at most PV_ANALYSE_NOALLOC_MAX_PAIRS (trial, block) pairs, i.e.
 * tdms * floor(nsamp / 2^bin_pow2) <= 1,048,576, about 12.6 MB; larger calls
 * return PV_ERR_ARG and a message naming the limit.  It calls no cudaMalloc,
 * cudaFree or allocating library routine.
 *
 * The first call on each device looks up the array's device address with
 * that device current; make that first call before any stream capture.  The
 * address is kept for the life of the process: the entry point assumes the
 * device's primary context (the one the CUDA runtime uses) and no
 * cudaDeviceReset between calls, after which the array would live at
 * another address.
 * Every call on a device shares the one array, so calls that overlap on the
 * GPU (other streams, other host threads) race and corrupt each other's
 * results; serialise them.  Nothing in the array needs clearing between
 * calls: each launch writes everything it reads. */
#define PV_ANALYSE_NOALLOC_MAX_PAIRS (1 << 20)
int pv_analyse_noalloc(const float* d_data, long long ld, int tdms, int nsamp, float threshold,
                       float rms, int bin_pow2, pv_event* d_events, long long cap,
                       long long* h_count, void* stream);

/* ------------------------------------------------------------------------
 * A2/A3 PPFChanneliser (lib/src/PPFChanneliser.cpp:29-290,
 * lib/src/PolyphaseCoefficients.cpp:77-364), A4 StokesGenerator
 * (lib/src/StokesGenerator.cpp:40-108), A5 StokesIntegrator
 * (lib/src/StokesIntegrator.cpp:32-119)
 * ---------------------------------------------------------------------- */

#define PV_WINDOW_HAMMING 0
#define PV_WINDOW_BLACKMAN 1
#define PV_WINDOW_GAUSSIAN 2
#define PV_WINDOW_KAISER 3

/* filter@filterWindow name -> PV_WINDOW_* (-1 and an error for others). */
int pv_window_from_name(const char* name);
/* PolyphaseCoefficients::genereateFilter: h_coeffs[t*nchan + c] (double). */
int pv_fir_coefficients(int ntaps, int nchan, int window, double* h_coeffs);

/* A channeliser with its per-(subband, polarisation) tap history on the
 * device.  nchan (outputChannelsPerSubband) is 1 or even, up to 1024
 * (PPFChanneliser.cpp:42-44): powers of two take a radix-2 FFT, other even
 * counts a direct DFT, and one channel passes the time series through
 * unfiltered (PPFChanneliser.cpp:108-131).  h_coeffs [ntaps][nchan] float,
 * or NULL to design them for `window` as the reference does (then converted
 * to float). */
typedef struct pv_ppf pv_ppf;
int pv_ppf_create(pv_ppf** ppf, int nchan, int ntaps, int window, const float* h_coeffs);
void pv_ppf_destroy(pv_ppf* ppf);
int pv_ppf_coefficients(const pv_ppf* ppf, float* h_out);
/* Forgets the tap history (next call starts from zeros, as a new module). */
int pv_ppf_reset(pv_ppf* ppf);
/* PPFChanneliser::run: d_in complex float [nsub][npol][nblocks*nchan]
 * (TimeSeriesDataSetC32, nTimesPerBlock = nchan); d_out complex float
 * [nblocks][nsub][npol][nchan] (SpectrumDataSetC32). */
int pv_ppf_run(pv_ppf* ppf, const float* d_in, int nsub, int npol, int nblocks, float* d_out,
               void* stream);
/* Fused PPF + Stokes + integration (dual polarisation): d_in as pv_ppf_run,
 * or raw int16 complex samples when in_int16; d_stokes receives
 * [nblocks/window][nsub][nstokes][nchan/bin] (SpectrumDataSetStokes after
 * StokesIntegrator); *nu_out the number of integrated samples. */
int pv_channelise(pv_ppf* ppf, const void* d_in, int in_int16, int nsub, int nblocks,
                  int nstokes, int window, int bin, float* d_stokes, int* nu_out, void* stream);
/* StokesGenerator::run: complex [nt][nsub][2][nchan] -> float
 * [nt][nsub][nstokes][nchan], nstokes 1 (I) or 4 (I,Q,U,V). */
int pv_stokes(const float* d_spectra, int nt, int nsub, int nchan, int nstokes, float* d_out,
              void* stream);
/* StokesIntegrator::run: [nt][nsub][npol][nchan] -> [nt/window][nsub][npol][nchan/bin]
 * (window reduced to nt when larger, remainders dropped). */
int pv_integrate(const float* d_in, int nt, int nsub, int npol, int nchan, int window, int bin,
                 float* d_out, int* nu_out, void* stream);

/* ------------------------------------------------------------------------
 * A6 RFI_Clipper (lib/src/RFI_Clipper.cpp:22-573) with BandPass,
 * BandPassAdapter and BinMap
 * ---------------------------------------------------------------------- */

/* bp_text is the BandPassData file's contents (BandPassAdapter format).
 * Arguments follow the XML: channelRejectionRMS, spectrumRejectionRMS,
 * History@maximum, zeroDMing@active, computeRMSfromMean@active,
 * Band@matching, and the element's active attribute. */
typedef struct pv_rfi pv_rfi;
int pv_rfi_create(pv_rfi** rfi, const char* bp_text, float channel_rejection_rms,
                  float spectrum_rejection_rms, int history, int zero_dming,
                  int compute_rms_from_mean, int band_matching, int active);
void pv_rfi_destroy(pv_rfi* rfi);
/* RFI_Clipper::run in place on device Stokes [nt][nsub][npol][nchan]
 * (statistics from pol 0).  d_flags (optional, [nt][nsub*nchan] bytes):
 * bit 0 channel clipped, bit 1 spectrum clipped.  The reference's weights
 * stay 1 (RFI_Clipper.cpp:143,332). */
int pv_rfi_run(pv_rfi* rfi, float* d_data, int nt, int nsub, int npol, int nchan,
               unsigned char* d_flags, void* stream);
/* [meanRunAve, rmsRunAve, bandpass mean, bandpass rms, bandpass offset,
 *  stats counter, bad spectra, mean history size, rms history size,
 *  unfilled last-good channels]; synchronous. */
int pv_rfi_state(pv_rfi* rfi, double* h_out10);
/* The rebinned bandpass model the first run used (host copy). */
int pv_rfi_bandpass(pv_rfi* rfi, float* h_out, int nbins);
/* The bandpass as RFI_Clipper::bandPass() holds it after the last spectrum
 * (lib/src/RFI_Clipper.cpp:562-563 setMean/setRMS, lib/BandPass.h:43-70):
 * h_out[nbins] its currentSet() (NULL: skipped), h_stats4 [mean, rms,
 * median, params()[0]].  Synchronous. */
int pv_rfi_bandpass_current(pv_rfi* rfi, float* h_out, int nbins, float* h_stats4);
/* The number of FP32 partial sums of the clipper's channel reductions for a
 * band of nbins channels (256, 512 or 1024): partial p sums channels p,
 * p + parts, ... in order. */
int pv_rfi_parts(int nbins);
/* How pv_rfi_run spreads a band over the GPU (no counterpart in the
 * reference, whose clipper is one CPU thread): 0 one CTA of `parts`
 * threads; 1 (the default) bands of 1024 partials over a cluster of 4 CTAs
 * of 256 threads; 2 bands of 512 or 1024 partials over clusters of 128-thread
 * CTAs.  Every choice computes the same partial sums, so flags and outputs
 * are identical. */
int pv_rfi_set_split(pv_rfi* rfi, int split);

/* ------------------------------------------------------------------------
 * One beam's device-resident chain, in the order of DedispersionPipeline::run
 * (src/pipelines/udpstream/src/DedispersionPipeline.cpp:96-174) with the
 * StokesIntegrator of UdpBFPipeline (UdpBFPipeline.cpp:80-92):
 * PPF -> Stokes I -> integrate -> RFI_Clipper -> DedispersionModule ->
 * DedispersionAnalyser, with the PPF tap history, the RFI state and the
 * per-channel delay ring kept on the device between chunks.
 * ---------------------------------------------------------------------- */
typedef struct {
    int nsub;           /* subbands */
    int nchan_sub;      /* PPFChanneliser outputChannelsPerSubband */
    int ntaps;          /* filter@nTaps */
    int window;         /* filter@filterWindow, PV_WINDOW_* */
    int int_time;       /* StokesIntegrator integrateTimeBins */
    int int_chan;       /* StokesIntegrator integrateFrequencyChannels */
    double fch1;        /* frequency of filterbank channel 0 (MHz) */
    double foff;        /* filterbank channel width (MHz; > 0 ascending) */
    double tsamp;       /* filterbank sample time (s) */
    int tdms;           /* dedispersionSamples */
    float dm_low;       /* dedispersionMinimum */
    float dm_step;      /* dedispersionStepSize */
    int chunk;          /* filterbank samples per chunk (= dedispersed samples per chunk) */
    float threshold;    /* detectionThreshold@in_sigma */
    int bin_pow2;       /* power2ForBinning */
    long long event_capacity; /* events kept per chunk (0: 2^20) */
    const char* bp_text;      /* RFI_Clipper BandPassData contents */
    float cr, sr;             /* channelRejectionRMS, spectrumRejectionRMS */
    int history;              /* History@maximum */
    int zero_dming, rms_from_mean, band_matching, rfi_active;
    int debug_taps;           /* keep the pre-RFI filterbank of the last chunk */
    int timing;               /* record CUDA events at the stage boundaries */
    int prefilled;            /* the delay ring starts as `lag` chunks of silence (zeros), so
                                 a window is dedispersed from the first chunk on; logical
                                 sample 0 is then the start of that silence and the first
                                 chunk's data starts at lag*chunk.  0: the reference's
                                 behaviour, the first window waits for lag+1 chunks. */
    int udp_packet_bytes;     /* > 0: a chunk is LOFAR UDP packets (pv_udp_config layout:
                                 16-byte header, [subband][16 samples][2 pols] complex int16,
                                 padded to this size; 16 + udp_subbands*128 for variable-size
                                 packets, 8148 for fixed), read by the channeliser in place
                                 of pv_udp_unpack's int16 voltages.  Needs 16, 32 or 64
                                 channels per subband and 8 taps. */
    int udp_subbands;         /* subbands per packet; the nsub / udp_subbands packet streams
                                 of a chunk follow each other, each chunk*int_time*nchan_sub/16
                                 packets long.  pv_beam_input_bytes is then the packet bytes
                                 of a chunk, and the in_int16 arguments do not apply. */
} pv_beam_config;

typedef struct pv_beam pv_beam;
int pv_beam_create(pv_beam** beam, const pv_beam_config* config);
void pv_beam_destroy(pv_beam* beam);
/* Bytes of one chunk of voltages: nsub x 2 pols x chunk*int_time*nchan_sub
 * complex samples of int16 (4 bytes) or float (8 bytes), layout
 * [sub][pol][sample] (TimeSeriesDataSetC32 order). */
long long pv_beam_input_bytes(const pv_beam* beam, int in_int16);
/* Processes one chunk from device (or host) memory, asynchronously. */
int pv_beam_process(pv_beam* beam, const void* d_voltages, int in_int16, void* stream);
int pv_beam_process_host(pv_beam* beam, const void* h_voltages, int in_int16, void* stream);
/* Events of the last dedispersed window (synchronises the stream): total
 * count including the dummy, the first sample of the window (-1 while the
 * ring is still filling), and up to cap events copied to h_events. */
int pv_beam_events(pv_beam* beam, pv_event* h_events, long long cap, long long* h_count,
                   long long* h_first_sample, void* stream);
/* [dedispersion channels, max delay, lag in chunks, ring samples, inverted,
 *  chunks processed, last window, ring bytes] */
int pv_beam_info(const pv_beam* beam, long long* h_info8);
/* Device time (ms) of the last dedispersed chunk's stages: channelise, RFI,
 * ring write, dedisperse, analyse (needs timing = 1; synchronises). */
int pv_beam_stage_ms(pv_beam* beam, float* h_ms5);
/* Saved state.  A beam's stream state is the PPF tap history per subband and
 * polarisation (the FIR buffer of PPFChanneliser, lib/PPFChanneliser.h:
 * 115-121), the clipper's running averages, history buffers and last good
 * spectrum (lib/RFI_Clipper.h:51-64) and the delay ring.  No reference
 * function saves it: the reference's modules keep it in memory for the life
 * of the pipeline.  Saving it lets a stream move to another process or GPU,
 * or restart, and continue bit for bit: a beam of the same configuration
 * that loads the state of a beam after chunk k and then processes chunk k+1
 * gives the windows and events the first beam gives.  The state is host
 * memory of pv_beam_state_size bytes (the ring dominates: channels x ring
 * samples x 4 bytes).  Save synchronises the stream; load synchronises too,
 * rejects a state of another configuration with PV_ERR_CONFIG, and leaves the
 * beam with no window read yet (pv_beam_events reports first sample -1
 * until the next window). */
long long pv_beam_state_size(const pv_beam* beam);
int pv_beam_state_save(pv_beam* beam, void* h_state, long long cap, void* stream);
int pv_beam_state_load(pv_beam* beam, const void* h_state, long long bytes, void* stream);
/* Device views of the last chunk's filterbank (after RFI), its pre-RFI copy
 * (debug_taps), the dedispersed window [tdms][chunk] and the ring. */
int pv_beam_buffers(const pv_beam* beam, float** d_filterbank, float** d_filterbank_raw,
                    float** d_dedispersed, float** d_ring);

/* ------------------------------------------------------------------------
 * Batched beams (the serving form).  No counterpart in the reference, whose
 * pipelines run one beam per process: many beams, each configured as for
 * pv_beam_create, advance one chunk per step, every stage of all beams in a
 * few launches (one persistent dedispersion launch over every beam's DM x
 * time tiles), optionally replayed from one captured CUDA graph.  A beam's
 * events equal those of the same beam run alone through pv_beam.
 * Restrictions: every beam has the same chunk (a multiple of 16 spectra), 8
 * PPF taps, 16, 32 or 64 channels per subband, int_chan = 1 and an int_time
 * dividing 256; input is complex int16.
 * ------------------------------------------------------------------------ */
typedef struct pv_batch pv_batch;
#define PV_BATCH_TUNE 1   /* autotune the dedispersion DM x time tile shape */
#define PV_BATCH_GRAPH 2  /* capture one step as a CUDA graph, replay it per step */
#define PV_BATCH_TIMING 4 /* record stage times of every step */
#define PV_BATCH_PIPELINED 8 /* dedisperse a beam's window in its step after the chunk that
                                completes it, beside that step's channeliser and clippers
                                (rings one chunk longer) */
#define PV_BATCH_STORE_F16 16 /* delay rings hold FP16 samples (sums stay FP32) */
#define PV_BATCH_STORE_U8 32  /* delay rings hold uint8 codes q with a per-channel FP32 scale and
                                 offset: the sample is (q - 128) * scale + offset, scale = 6 sigma
                                 / 127.  With the clipper and zero-DMing its output has zero
                                 mean and unit RMS: sigma = 1, offset 0.  Otherwise the offset is
                                 the median and sigma the median absolute deviation x 1.4826 of
                                 the first chunk in which the channel varies (until then the
                                 channel's samples are stored as its offset) */
/* How the clippers spread over the GPU.  Every choice computes the same
 * partial sums, so the flags and outputs are identical.  By default a
 * pipelined batch gives each beam's clipper one CTA (the clippers share the
 * GPU with the dedispersion) and an unpipelined batch spreads beams of more
 * than 4096 channels over a cluster of 4 CTAs (the clippers run alone). */
#define PV_BATCH_RFI_ONE_CTA 64   /* one CTA per beam */
#define PV_BATCH_RFI_CLUSTER8 128 /* beams of more than 1024 channels on clusters of 128-thread CTAs
                                     (4 CTAs up to 4096 channels, 8 beyond) */
#define PV_BATCH_RFI_CLUSTER4 0x10000 /* beams of more than 4096 channels on a cluster of 4 CTAs */
#define PV_BATCH_VARIANTS 9            /* dedispersion tile variants (4 to 8: FP32 rings only) */
#define PV_BATCH_VARIANT(v) ((v) << 8) /* without PV_BATCH_TUNE: tile variant 0..8 */
#define PV_BATCH_VARIANT_OF(flags) ((((flags) >> 8) & 0xff) % PV_BATCH_VARIANTS)
int pv_batch_create(pv_batch** batch, const pv_beam_config* configs, int nbeams, int flags);
void pv_batch_destroy(pv_batch* batch);
#define PV_BATCH_HOST_EVENTS 65536 /* events per beam per step kept in host memory */
/* The device buffer beam's voltages are read from at the next step
 * (pv_beam_input_bytes(.., 1) bytes, [sub][pol][sample] complex int16).
 * Steps alternate between two buffer sets, so ask again before every step. */
int pv_batch_input(pv_batch* batch, int beam, void** d_voltages, long long* bytes);
/* The input buffer of a beam's chunks of one parity (0: its 1st, 3rd, ...
 * chunk; 1: its 2nd, 4th, ...): a caller that feeds the same chunk every
 * step fills both once. */
int pv_batch_input_parity(pv_batch* batch, int beam, int parity, void** d_voltages, long long* bytes);
/* One step from the input buffers, asynchronously.  h_active[beam] != 0
 * (h_active NULL: every beam) marks the beams that have a chunk this step;
 * the others keep their state and skip every stage (a serving loop's
 * continuous batching).  A beam dedisperses a window in the step whose chunk
 * completes it; pipelined, in the next step (whether or not the beam has a
 * chunk then).  At most two steps are in flight: issuing a step waits for
 * the step two back. */
int pv_batch_run(pv_batch* batch, const unsigned char* h_active, void* stream);
/* Copies h_voltages[beam] of the active beams (host, page-locked for speed)
 * to their input buffers on the batch's own copy stream, then runs the step
 * on `stream` once the copies land.  Returns at once: the copies of step
 * k+1 overlap the computation of step k. */
int pv_batch_run_host(pv_batch* batch, const void* const* h_voltages, const unsigned char* h_active,
                      void* stream);
/* Events of one beam at one of the last two issued steps (step >= 0: that
 * step; -1: the last issued, -2: the one before), as pv_beam_events: total count including the dummy, the window's
 * first sample (-1: the beam dedispersed no window in that step) and up to
 * cap events (at most PV_BATCH_HOST_EVENTS) copied to h_events.  Waits for
 * that step only, so the next step may already be running. */
int pv_batch_events(pv_batch* batch, int beam, long long step, pv_event* h_events, long long cap,
                    long long* h_count, long long* h_first_sample);
/* [dedispersion channels, max delay, lag in chunks, ring samples, inverted,
 *  chunks in the ring (prefilled silence included), last window dedispersed
 *  (-1: none), ring bytes] after the steps issued. */
int pv_batch_info(const pv_batch* batch, int beam, long long* h_info8);
/* Dedispersion tiling: [variant, time tile, channels per stage, stages,
 * slot floats, tiles, CTAs, shared bytes], the DM tile height of every beam,
 * the autotuner's time (ms) of each of the PV_BATCH_VARIANTS variants (-1:
 * not timed or not usable) and the kernels one graph replay launches (0
 * without a graph).  Any may be NULL.  Variants 0-3 give each trial of a
 * DM tile one warp (one shared-memory word per add); variants 4 to 8 give
 * each warp two adjacent trials that share the words they both read
 * (6 to 8 read from registers shift differences up to 15 instead of 32,
 * 7 and 8 with 14 adding warps instead of 12). */
int pv_batch_tiles(const pv_batch* batch, int* h_shape8, int* h_dms, float* h_tune_ms,
                   long long* h_graph_kernels);
/* Device time (ms) of the last step's stages (PV_BATCH_TIMING): channelise,
 * RFI, ring write, dedisperse, analyse (pipelined: the last two run
 * concurrently with the first three). */
int pv_batch_stage_ms(pv_batch* batch, float* h_ms5);
int pv_batch_buffers(const pv_batch* batch, int beam, float** d_filterbank, float** d_dedispersed,
                     float** d_ring);
/* Starts a new stream in slot `beam` of the batch: the slot's ring (prefilled
 * silence again when configured so), PPF history, clipper state and window
 * go back to those of a new beam of the same configuration, so a serving
 * loop gives a drained stream's slot, and its device memory, to the next
 * stream of that configuration without rebuilding the batch or its graph.
 * Waits for the issued steps; the slot's next step is the new stream's
 * first chunk.  (A pelican pipeline gets the same by creating its modules
 * again.) */
int pv_batch_reset_beam(pv_batch* batch, int beam, void* stream);
/* 1 if step `step` (one of the steps issued) has finished on the device, 0 if not. */
int pv_batch_step_done(const pv_batch* batch, long long step);
/* Device bytes one beam of this configuration takes in a batch created with
 * `flags` (ring, input buffers, filterbank, window, events, scratch): the
 * admission cost of a serving loop under an HBM budget. */
long long pv_batch_footprint(const pv_beam_config* config, int flags);

/* ---- Serving loop ---------------------------------------------------------
 * No counterpart in the reference, whose pipelines run one beam per process
 * (pipelines/udpstream/src/DedispersionPipeline.cpp:96-174).  pv_serve runs
 * streams of chunks from many beams through the batched engine in real time:
 * a chunk is queued as sub-chunks of one step (the configuration's chunk)
 * each; streams are admitted under an HBM budget (pv_batch_footprint); a
 * stream that arrives takes at once the slot of a drained stream of the same
 * configuration in a running cohort (pv_batch_reset_beam), the others are
 * admitted first fit every admit_every seconds as a new cohort (one batch on
 * its own CUDA stream: the steps of all cohorts overlap); every step of a
 * cohort takes one sub-chunk of each beam with one queued (continuous
 * batching), at most max_inflight steps in flight; a cohort whose streams
 * have drained is released, its memory returned, once a waiting stream needs
 * the memory or after it has lingered idle `linger` seconds.  A chunk's latency runs from its arrival to the end of
 * the step that processed its last sub-chunk.  PV_SERVE_FIFO1 is the plain
 * per-chunk path: one pv_beam per stream, the oldest queued sub-chunk alone,
 * its events read back before the next. */
#define PV_SERVE_BATCH 0
#define PV_SERVE_FIFO1 1
typedef struct {
    double budget_bytes;  /* device memory the admitted beams may take */
    int policy;           /* PV_SERVE_BATCH or PV_SERVE_FIFO1 */
    int batch_flags;      /* pv_batch_create flags of every cohort (PV_BATCH_GRAPH, PIPELINED, STORE_*) */
    int max_inflight;     /* steps in flight per cohort, 1 or 2 (0: 2) */
    double admit_every;   /* seconds between admission rounds of new cohorts */
    double horizon;       /* stop after this many seconds (0: when every chunk is served) */
    int reuse_slots;      /* give a drained stream's slot to a waiting stream of the same configuration */
    double linger;        /* seconds a drained cohort is kept for a stream of its configuration when no
                             waiting stream needs its memory */
} pv_serve_config;
typedef struct {
    int nchunks;               /* chunks of the stream */
    const double* arrivals;    /* their arrival times, seconds from the start, ascending */
    const int* sizes;          /* their sizes in spectra, multiples of the configuration's chunk */
    const void* h_voltages;    /* page-locked int16 voltages of one sub-chunk (pv_beam_input_bytes),
                                  the stream's receive buffer, copied in for every sub-chunk */
    double units_per_spectrum; /* DM trials x channels: the work one spectrum brings */
} pv_serve_stream;
typedef struct {
    long long chunks, chunks_done, cohorts, slot_reuses, steps;
    int max_concurrent_beams;
    double wall_s, units, throughput; /* DM-trial*chan*samples per second of wall time */
    double latency_p50, latency_p99, latency_max;             /* seconds from arrival to processed */
    double latency_admitted_p50, latency_admitted_p99;        /* chunks arriving after admission */
    double latency_over_duration_p50, latency_over_duration_p99; /* latency / the chunk's duration */
    double within_real_time;                                  /* share of chunks with latency < duration */
    double admission_wait_p50, admission_wait_p99;            /* first arrival to admission */
    double peak_footprint_bytes;
} pv_serve_stats;
/* Hooks that replace the GPU engine and the wall clock (tests drive the loop
 * on the CPU with them).  open returns a cohort handle for n streams (NULL:
 * failure); step returns a step id (< 0: failure); done: 1 once that step
 * has finished; reset_slot: PV_OK once slot `slot` serves stream `stream`. */
typedef struct {
    void* ctx;
    long long (*footprint)(void* ctx, const pv_beam_config* config);
    void* (*open)(void* ctx, const pv_beam_config* configs, const int* streams, int n);
    long long (*step)(void* ctx, void* cohort, const unsigned char* active, int n);
    int (*done)(void* ctx, void* cohort, long long step);
    int (*reset_slot)(void* ctx, void* cohort, int slot, int stream);
    void (*close)(void* ctx, void* cohort);
    double (*clock)(void* ctx);           /* seconds (NULL: the wall clock) */
    void (*sleep)(void* ctx, double seconds);
    /* events of a finished step's slot: the total count, *first the window's first
       sample (-1: none this step), up to cap events copied to out (NULL: no output) */
    long long (*events)(void* ctx, void* cohort, long long step, int slot, pv_event* out, long long cap,
                        long long* first);
} pv_serve_engine;
/* Where the events of every dedispersed window go (the pipeline's
 * "DedispersionDataAnalysis" stream): called from pv_serve's thread for each
 * window of each stream, in order, with the window's first sample in the
 * stream, up to PV_BATCH_HOST_EVENTS events and their total (dummy first). */
typedef struct {
    void* ctx;
    void (*events)(void* ctx, int stream, long long first_sample, const pv_event* events, long long n,
                   long long total);
} pv_serve_output;
/* Serves the streams (configs[i] is stream i's beam) until every chunk is
 * processed or the horizon passes, then fills *stats.  engine NULL: the
 * library's batched engine (or pv_beam per stream for PV_SERVE_FIFO1). */
int pv_serve(const pv_serve_config* config, const pv_beam_config* configs, const pv_serve_stream* streams,
             int nstreams, const pv_serve_engine* engine, const pv_serve_output* output, pv_serve_stats* stats);

/* ---- LOFAR UDP ingest (AdapterTimeSeriesDataSet) -------------------------
 * Replaces AdapterTimeSeriesDataSet::deserialise/_checkData/_readData
 * (lib/src/AdapterTimeSeriesDataSet.cpp:78-293).  Fields are the adapter's
 * XML options (:37-45).  A chunk is packets_per_chunk packets of a 16-byte
 * header (lib/LofarUdpHeader.h:25-35) and subband-major data
 * [subband][time][pol] of complex int8 or int16, padded to 8148 bytes when
 * fixed_size_packets. */
typedef struct {
    int fixed_size_packets; /* <fixedSizePackets value="true"/> */
    int sample_bits;        /* <dataBitSize value="16"/>: 8 or 16 */
    int packets_per_chunk;  /* <udpPacketsPerIteration value=.../> */
    int samples_per_packet; /* <samplesPerPacket value="16"/> */
    int nchan;              /* <outputChannelsPerSubband value=.../>: samples per time block */
    int nsub;               /* <subbandsPerPacket value=.../> */
    int npol;               /* <nRawPolarisations value="2"/> (16-bit data: 2) */
    int clock_mhz;          /* <clock value="200"/> */
} pv_udp_config;
#define PV_UDP_OUT_C32 0 /* complex float [sub][pol][block][nchan]: TimeSeriesDataSetC32 */
#define PV_UDP_OUT_I16 1 /* complex int16, same order: the station format pv_channelise,
                            pv_beam_process and pv_batch take with in_int16 = 1 */
/* _checkData (AdapterTimeSeriesDataSet.cpp:152-191): packet bytes and time
 * blocks of a chunk of chunk_bytes; PV_ERR_CONFIG with the reference's message. */
int pv_udp_check(const pv_udp_config* config, long long chunk_bytes, long long* h_packet_bytes,
                 int* h_nblocks);
/* _readData (:209-282) for every packet of the device chunk, into d_out
 * (nsub*npol*packets*samples complex elements of out_type). */
int pv_udp_unpack(const pv_udp_config* config, const void* d_chunk, long long chunk_bytes,
                  void* d_out, int out_type, void* stream);
/* The chunk's LOFAR time stamp (seconds) and block rate (seconds per sample)
 * from its first packet's header (:107-118). */
int pv_udp_time(const pv_udp_config* config, const void* h_packet, double* h_timestamp,
                double* h_block_rate);

/* ---- ALFABURST spectrometer packets: ABDataAdapter ------------------------
 * ABDataAdapter::deserialise (lib/src/ABDataAdapter.cpp:14-173), the input of
 * ABPipeline (pipelines/udpstream/src/ABPipeline.cpp:56-140).  A packet is an
 * 8-byte header (bytes 0-5: the integration count, most significant byte
 * first; byte 6: the spectral quarter; byte 7: the beam) and `channels`
 * records of four big-endian 16-bit pseudo-Stokes values (XX, YY, XY re,
 * XY im): 8 + 8 * channels bytes. */
typedef struct pv_ab_config {
    int packets_per_spectrum; /* <spectrum packets> */
    int channels;             /* <packet channels> */
    int samples_per_packet;   /* <packet samples>; 0 (absent) counts as 1 */
    float tsamp;              /* <samplingTime seconds> */
} pv_ab_config;
/* What the adapter carries from chunk to chunk; zero it before the first. */
typedef struct pv_ab_state {
    long long seen;              /* packets read so far */
    unsigned long long count0;   /* the first packet's integration count */
    double last_time;            /* the previous packet's time */
} pv_ab_state;
/* The header pass over one chunk in host memory (:68-150).  The chunk holds
 * bytes / packet size packets and the blob (packets / packets_per_spectrum) *
 * samples_per_packet spectra (*h_nblocks).  Each packet whose spectral
 * quarter is packets_per_spectrum - 3 fills the next spectrum: h_index
 * receives the packets' indices (at most min(cap, *h_nblocks); *h_nspectra of
 * them).  A packet's time is (count - count0) * tsamp, count0 being 0 for the
 * very first packet and that packet's count afterwards; *h_timestamp is the
 * chunk's last packet's time and *h_gaps counts the packets more than tsamp
 * after the previous one (the reference's "FATAL!" lines). */
int pv_ab_headers(const pv_ab_config* config, pv_ab_state* state, const void* h_chunk, long long bytes,
                  int* h_index, long long cap, long long* h_nspectra, long long* h_nblocks,
                  double* h_timestamp, long long* h_gaps);
/* The data pass on the device: spectrum k of d_out [nblocks][channels] float
 * is XX + YY (unsigned 16-bit) of packet d_index[k] for k < nspectra, and 0
 * for the rest. */
int pv_ab_unpack(const pv_ab_config* config, const void* d_chunk, long long bytes, const int* d_index,
                 long long nspectra, long long nblocks, float* d_out, void* stream);

/* ---- Outputs: sigproc filterbank and event text --------------------------
 * SigprocStokesWriter (lib/src/SigprocStokesWriter.cpp:15-293) and
 * DedispersionDataAnalysisOutput (lib/src/DedispersionDataAnalysisOutput.cpp:
 * 18-112).  Header values are the writer's members as it writes them
 * (floats widened to double); the shim's SigprocStokesWriter derives them
 * from the XML options. */
typedef struct {
    int machine_id;        /* <MachineID value="9"/> */
    int telescope_id;      /* <TelescopeID value="0"/> */
    int nchans;            /* channels per spectrum written */
    int nbits;             /* <dataBits value="32"/>: 32 or 8 */
    int nifs;              /* <params nPolsToWrite="1"/> */
    double src_raj, src_dej, fch1, foff, tsamp;
    double tstart;         /* MJD (pv_sigproc_mjd) */
    char source_name[80];  /* NUL-terminated */
} pv_sigproc_params;
/* The header bytes (HEADER_START .. HEADER_END, :118-140) into h_buf;
 * *h_len is the size needed (PV_ERR_ARG when cap is smaller). */
int pv_sigproc_header(const pv_sigproc_params* params, char* h_buf, long long cap, long long* h_len);
/* MJD of a LOFAR (Unix) time stamp: (t - 2011-01-01 00:00 UTC) / 86400 + 55562
 * (:120-128; the reference's mktime takes the host's time zone). */
double pv_sigproc_mjd(double lofar_timestamp);
/* The data block of nt spectra (:195-234) on the device: d_stokes is
 * SpectrumDataSetStokes float [t][sub][pol][chan]; d_out receives, per t and
 * written polarisation p < npols_write, subbands then channels in descending
 * order, as float (nbits 32) or one byte rint((min(x, crop_max) - crop_min) *
 * 255 / (crop_max - crop_min)), 0 below crop_min (nbits 8, :288-293). */
int pv_sigproc_pack(const float* d_stokes, int nt, int nsub, int npol, int nchan, int npols_write,
                    int nbits, float crop_min, float crop_max, void* d_out, void* stream);
/* The text DedispersionDataAnalysisOutput::sendStream writes for one analysed
 * buffer (:80-112): a line "mjd,   dm, snr, binFactor" per event after the
 * first, then "# Written buffer :<dump_index> | MJDstart: ... Done".  Times
 * are start_timestamp + (t + first_sample) * block_rate of the buffer's first
 * input blob; dm = dm_low + dm_step * index; snr = value / (rms *
 * sqrt(binFactor)).  *h_len is the size needed. */
int pv_events_text(const pv_event* h_events, long long n, double start_timestamp, double block_rate,
                   long long first_sample, double dm_low, double dm_step, float rms, int dump_index,
                   char* h_buf, long long cap, long long* h_len);
/* The FRATS trigger TriggerOutput::_convertToTrigger_FRATS sends for one
 * analysed buffer (lib/src/TriggerOutput.cpp:151-183).  When the buffer holds
 * at least min_events events (the analyser's first event counts), the event of
 * largest snr = value / (rms * sqrt(binFactor)) in float (above 0; the first
 * of equals) gives, if snr >= snr_threshold, the message
 *   artemis:<station>##ID:<id_root><message_number>##cFreqMHz:<cfreq_mhz>
 *   ##beamRA:<beam_ra>##beamDec:<beam_dec>##eTime:<time %.9f>##eDM:<dm %.3f>
 *   ##eSNR:<snr %.2f>
 * (one line; fields left-padded with '0' to 4, 10, 10, 9, 20, 9 and 6
 * characters, never cut).  Time and dm as in pv_events_text.  *h_len is the
 * message size, 0 when the buffer raises no trigger; h_buf may be null for a
 * size query. */
int pv_trigger_message(const pv_event* h_events, long long n, double start_timestamp, double block_rate,
                       long long first_sample, double dm_low, double dm_step, float rms, int min_events,
                       float snr_threshold, const char* station, const char* id_root, int message_number,
                       const char* cfreq_mhz, const char* beam_ra, const char* beam_dec, char* h_buf,
                       long long cap, long long* h_len);
/* ---- BandPassRecorder (lib/src/BandPassRecorder.cpp:22-190) ---------------
 * Options: <requiredSamples value="20000"/>, <fitParmaters coefficients="3"/>,
 * <Band startFrequency=.. endFrequency=../>.  The integrated Stokes-I
 * spectrum is summed on the device; the polynomial fit with 2-sigma
 * trimming of high channels is made on the host once required_samples
 * spectra have been added (the reference's intent: its own LAPACK call cannot
 * run). */
typedef struct pv_bandpass_recorder pv_bandpass_recorder;
int pv_bandpass_recorder_create(pv_bandpass_recorder** recorder, long long required_samples, int ncoeffs,
                                float start_freq, float end_freq);
void pv_bandpass_recorder_destroy(pv_bandpass_recorder* recorder);
/* BandPassRecorder::run: adds polarisation 0 of d_stokes [t][sub][pol][chan].
 * Returns 1 when the fit is ready (the stream is synchronised), 0 while
 * more spectra are needed, or an error.  The next call after a fit starts a
 * new integration. */
int pv_bandpass_recorder_add(pv_bandpass_recorder* recorder, const float* d_stokes, int nt, int nsub,
                             int npol, int nchan, void* stream);
/* The fit: ncoeffs coefficients of f^0..f^(n-1), the RMS of the cleaned mean
 * spectrum, the channels trimmed, and the .bp text (BandPassAdapter format,
 * lib/src/BandPassAdapter.cpp:30-108) that pv_rfi_create loads. */
int pv_bandpass_recorder_result(const pv_bandpass_recorder* recorder, float* h_coeffs, float* h_rms,
                                int* h_trimmed, char* h_bp_text, long long cap, long long* h_len);

/* The file header DedispersionDataAnalysisOutput writes when it opens a file (:66-70). */
#define PV_EVENTS_TEXT_HEADER \
    "# Generated by DedispersionDataAnalysisOutput\n# Events\n# ------\n# Time|Dm|Amplitude|BinFactor\n# ------\n"

#ifdef __cplusplus
}
#endif
#endif /* PV_H */
