// Internal (non-ABI) entry points shared between translation units.
#pragma once

#include <vector>

#include "pv_common.cuh"

// Element type of a batch's delay rings.
#define PV_STORE_F32 0
#define PV_STORE_F16 1
#define PV_STORE_U8 2

namespace pv {

// A batch beam's progress, device-resident.  The planning kernel at the start
// of every step sets `active` (a chunk of this beam is processed) and `sel` (a
// window of this beam is dedispersed, `window` its index); every batched
// kernel skips the beams it does not concern, and the last kernel of the step
// advances `written` and `done`.
struct BeamStep {
    long long written;  // logical chunks in the ring, prefilled silence included
    long long done;     // windows dedispersed so far
    long long base;     // prefilled chunks of silence
    long long window;   // window dedispersed this step (valid when sel)
    int lag;            // window w needs ring chunks w..w+lag
    int active, sel;
    int pad;
};

// One beam's share of a Stokes-I channeliser launch (chan_stokes_i_kernel).
struct ChanJob {
    const void* in;          // [sub][2][nblocks*N] short2 or float2 voltages
    const void* in_odd;      // read instead of `in` at odd device steps (null: always `in`)
    float2* hist[2];         // [sub][2][7][N]: hist[step & 1] is read (null: zeros), the other written
    const float* coeffs;     // [8][N]
    const float2* twiddle;   // [N/2] exp(-2 pi i k / N)
    float* out;              // [nu][sub][N] Stokes I
    long long warp_begin;    // first warp of this job in the launch
    int nsub, nblocks, window, nu, nranges;
    int beam;                // index into the batch's BeamStep array
    long long pkt_bytes;     // > 0: `in` holds LOFAR packets of this size (int16, 16 samples each)
    int pkt_nsub;            // subbands per packet; the nsub/pkt_nsub streams follow each other
};
bool chan_fast_supported(int nchan, int ntaps, int npol, int nstokes, int window, int bin, int nblocks);
// pv_channelise (Stokes I, int16 input) with the input in the LOFAR packet layout when
// pkt_bytes > 0 (the register channeliser only)
int channelise_stokes_i(pv_ppf* h, const void* d_in, int nsub, int nblocks, int window, int bin, float* d_stokes,
                        int* nu_out, long long pkt_bytes, int pkt_nsub, cudaStream_t s);
int chan_job_warps(ChanJob& job);  // sets nranges, returns the job's warp count
// bs == null: one job, always active, input `in`, history hist[0] -> hist[1].
// input: 0 complex float voltages, 1 int16 voltages, 2 int16 LOFAR packets (pkt_bytes of every job)
int launch_chan_fast(int nchan, int input, const ChanJob* d_jobs, const ChanJob& one, int njobs,
                     long long nwarps, const BeamStep* bs, cudaStream_t s);
// Saved state of one beam (pv_beam_state_*): the PPF tap history and the
// clipper's running state, as bytes in host memory.
long long ppf_state_bytes(const pv_ppf* h, int nsub, int npol);
int ppf_state_io(pv_ppf* h, int nsub, int npol, void* h_buf, bool save, cudaStream_t s);
long long rfi_state_bytes(const pv_rfi* h, int nbins);
int rfi_state_io(pv_rfi* h, int nbins, void* h_buf, bool save, cudaStream_t s);
int rfi_reset(pv_rfi* h, cudaStream_t s);
// coefficient [T][N] and twiddle [N/2] tables of a PPF handle
int ppf_tables(const pv_ppf* h, const float** d_coeffs, const float2** d_twiddle, int* nchan,
               int* ntaps);
// delay constants (device and host) and trial scaling of a dedispersion plan
int plan_tables(const pv_dedisp_plan* p, const float** d_dmshift, const float** h_dmshift,
                int* nchan, int* tdms, float* start, float* step);

// Batched dedispersion (dedisperse.cu): one beam's ring and window.
struct DdBeam {
    float* out;
    long long out_stride;
    const float* ring;               // elements of the batch's storage type
    long long row_stride, ring_len;  // in elements
    const float* d_dmshift;
    const float* scale;              // u8 storage: per-row scale (a byte q is (q-128)*scale+offset)
    const float* off_sum;            // u8 storage: sum of the rows' offsets
    const float* h_dmshift;
    int nchan, nout, tdms, chunk;
    float start, step;  // trial value = start + d*step, in samples per unit delay constant
    int uniform;        // u8 storage: every row has the scale scale[0] (codes summed as integers)
};
struct DdJob {
    float* out;
    long long out_stride;
    const float* ring;
    long long row_stride, ring_len;
    const float* dmshift;
    const float* scale;
    const float* off_sum;
    int nchan, nout, tdms, chunk, dms, beam;
    float start, step;
    int uniform;
};
struct DdTile {
    int job, d0, t0;
};
struct DdBatch;
// variant < 0 runs the autotuner over the DM x time tile variants; store: PV_STORE_*
int dd_batch_create(DdBatch** out, const DdBeam* beams, int n, int variant, int store, cudaStream_t s);
int dd_batch_launch(DdBatch* b, const BeamStep* bs, cudaStream_t s);
// Launches that share one tile queue: reset the queue once, then launch any
// number of `ctas`-CTA kernels (possibly on other streams) that drain it.
int dd_batch_reset(DdBatch* b, cudaStream_t s);
int dd_batch_launch_shared(DdBatch* b, const BeamStep* bs, int ctas, cudaStream_t s);
int dd_batch_grid(const DdBatch* b);
int dd_batch_status(const DdBatch* b, int* h_status);
int dd_batch_shape(const DdBatch* b, int* h8);
const std::vector<int>& dd_batch_dms(const DdBatch* b);
const int* dd_batch_status_word(const DdBatch* b);
const std::vector<float>& dd_batch_tune_ms(const DdBatch* b);
void dd_batch_destroy(DdBatch* b);

// Batched RFI clippers (rfi.cu).
struct RfiBatch;
// handles[i] null: beam i has no clipper; bs: the batch's BeamStep array (inactive beams skip);
// split: 0 one CTA per beam; 1 beams of more than 4096 channels on a cluster of 4 CTAs;
// 2 beams of more than 1024 channels on clusters of 128-thread CTAs
int rfi_batch_create(RfiBatch** out, pv_rfi* const* handles, float* const* data, const int* nsub,
                     const int* nchan, int n, int nt, const BeamStep* bs, int split, cudaStream_t s);
int rfi_batch_launches(const RfiBatch* b);  // number of classes (beams with one channel count), largest first
int rfi_batch_launch_one(RfiBatch* b, int k, cudaStream_t s);
int rfi_batch_ctas(const RfiBatch* b, int k);  // CTAs of class k (beams x CTAs per beam)
void rfi_batch_destroy(RfiBatch* b);

// Batched ring writes (buffer.cu): stokes [nt][nsub][1][nchan] of one beam.
struct RingJob {
    float* ring;
    long long row_stride, ring_len;
    const float* stokes;
    int nt, nsub, nchan, inverted;
    long long block_begin;  // first CTA of this job
    int beam;               // index into the BeamStep array: written chunks give the position
    float* scale;           // u8 rings: per-row scale (0 until the row is calibrated)
    float* offset;          // u8 rings: per-row offset
    float* off_sum;         // u8 rings: sum of the offsets
    long long cal_begin;    // first CTA of this job in the calibration launch
};
int ring_job_blocks(const RingJob& j);
int ring_cal_blocks(const RingJob& j);
// store: PV_STORE_* element type of the rings
int ring_write_batch(const RingJob* d_jobs, int njobs, long long nblocks, const BeamStep* bs,
                     int store, cudaStream_t s);
// u8 rings: scales and offsets of the rows not calibrated yet, from this
// step's chunk, and every beam's offset sum
int ring_calibrate_batch(const RingJob* d_jobs, int njobs, long long nblocks, const BeamStep* bs,
                         cudaStream_t s);

int ring_write_device(float* ring, long long row_stride, long long ring_len, long long pos,
                      const float* stokes, int nt, int nsub, int npol, int nchan, int inverted,
                      cudaStream_t s);

size_t analyse_scratch_bytes(int tdms, int nsamp, int bin_pow2);
int analyse_launch(const float* data, long long ld, int tdms, int nsamp, float threshold, float rms,
                   int bin_pow2, pv_event* ev, long long cap, long long* d_total, void* scratch,
                   cudaStream_t s);

}  // namespace pv

namespace pv {
// elem_bytes: 4 (float rings), 2 (half) or 1 (u8, cleared to the code 128)
int beam_create(pv_beam** out, const pv_beam_config* c, int extra_ring_chunks, int elem_bytes = 4);
}

// One beam's device-resident chain state (beam.cu); the batch engine reuses it.
struct pv_beam {
    pv_beam_config cfg{};
    pv_ppf* ppf = nullptr;
    pv_rfi* rfi = nullptr;
    pv_dedisp_plan* plan = nullptr;
    int nchan_fb = 0;        // filterbank channels per subband after integration
    int nbins = 0;           // dedispersion channels
    int inverted = 0;
    int max_shift = 0, lag = 0;
    long long ring_len = 0, row_stride = 0;
    float* d_ring = nullptr;
    float* d_fb = nullptr;       // [chunk][nsub][1][nchan_fb]
    float* d_fb_raw = nullptr;   // optional pre-RFI copy
    float* d_out = nullptr;      // [tdms][chunk]
    pv_event* d_events = nullptr;
    long long cap = 0;
    void* d_scratch = nullptr;
    long long* d_total = nullptr;
    long long* h_total = nullptr;  // pinned
    void* d_in = nullptr;          // staging for host input
    size_t in_bytes = 0;
    long long chunks = 0;
    long long window = -1;
    float rms = 0.0f;
    cudaEvent_t ev[6] = {};     // stage boundaries of the last chunk (timing mode)
    bool timed = false;
};
