// ALFABURST spectrometer ingest: chunks of spectrum packets -> SpectrumDataSetStokes.
//
// Replaces ABDataAdapter::deserialise (lib/src/ABDataAdapter.cpp:14-173), the
// adapter of ABPipeline (pipelines/udpstream/src/ABPipeline.cpp:56-140).  The
// spectrometer sends each spectrum as packets_per_spectrum packets ("spectral
// quarters"); a packet is an 8-byte header and `channels` records of four
// big-endian 16-bit pseudo-Stokes values (XX, YY, XY re, XY im).  The adapter
// keeps one quarter per spectrum (quarter packets_per_spectrum - 3) and
// writes Stokes I = XX + YY of its channels as one block of a one-subband,
// one-polarisation SpectrumDataSetStokes.
//
// The headers (integration counts, quarters, gaps) are a sequential scan on
// the host, as in the reference; the spectra are assembled on the GPU from
// the chunk copied in once.  Each thread takes one channel of one spectrum:
// one aligned 8-byte load of the record, two byte swaps and an add.
#include <algorithm>
#include <cstring>

#include "pv_internal.cuh"

namespace {

constexpr long long kAbHeaderBytes = 8;

long long packet_bytes(const pv_ab_config* c) { return kAbHeaderBytes + 8LL * c->channels; }

int check_config(const pv_ab_config* c, const char* who) {
    if (!c || c->packets_per_spectrum <= 0 || c->channels <= 0 || c->samples_per_packet < 0) {
        pv::set_error("%s: <spectrum packets>, <packet channels> must be positive", who);
        return PV_ERR_CONFIG;
    }
    return PV_OK;
}

long long blob_blocks(const pv_ab_config* c, long long packets) {
    const long long spp = c->samples_per_packet > 0 ? c->samples_per_packet : 1;
    return packets / c->packets_per_spectrum * spp;
}

__global__ void __launch_bounds__(256)
ab_unpack_kernel(const uint2* __restrict__ chunk, long long npackets, int channels, const int* __restrict__ index,
                 long long nspectra, long long nblocks, float* __restrict__ out) {
    const long long n = nblocks * channels;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const long long k = i / channels;
        const int c = (int)(i - k * channels);
        float v = 0.0f;
        if (k < nspectra) {
            const long long p = index[k];
            if (p >= 0 && p < npackets) {
                // record c of packet p: 8-byte units, the header first
                const unsigned w = chunk[p * (channels + 1) + 1 + c].x;  // XX, YY big-endian
                const unsigned xx = __byte_perm(w, 0u, 0x4401u), yy = __byte_perm(w, 0u, 0x4423u);
                v = (float)(xx + yy);
            }
        }
        out[i] = v;
    }
}

}  // namespace

extern "C" int pv_ab_headers(const pv_ab_config* c, pv_ab_state* st, const void* h_chunk, long long bytes,
                             int* h_index, long long cap, long long* h_nspectra, long long* h_nblocks,
                             double* h_timestamp, long long* h_gaps) {
    PV_TRY(check_config(c, "ABDataAdapter"));
    if (!st || (!h_chunk && bytes > 0) || bytes < 0 || !h_nspectra || !h_nblocks || !h_timestamp || !h_gaps ||
        cap < 0 || (!h_index && cap > 0)) {
        pv::set_error("pv_ab_headers: invalid arguments");
        return PV_ERR_ARG;
    }
    const long long psize = packet_bytes(c);
    const long long npk = bytes / psize;
    const long long nblocks = blob_blocks(c, npk);
    const unsigned keep = (unsigned)(c->packets_per_spectrum - 3);  // unsigned, as the reference compares
    const double tsamp = (double)c->tsamp;
    const auto* base = static_cast<const unsigned char*>(h_chunk);
    long long nsp = 0, gaps = 0;
    double t = 0.0;
    for (long long p = 0; p < npk; ++p) {
        const unsigned char* h = base + p * psize;
        unsigned long long count = 0;
        for (int b = 0; b < 6; ++b) count = (count << 8) | h[b];
        t = (double)(count - (st->seen ? st->count0 : 0ULL)) * tsamp;
        if (st->seen) {
            if (t - st->last_time > tsamp) ++gaps;
        } else {
            st->count0 = count;
        }
        if ((unsigned)h[6] == keep && nsp < nblocks) {
            if (nsp >= cap) {
                pv::set_error("pv_ab_headers: index capacity %lld below the chunk's spectra", cap);
                return PV_ERR_ARG;
            }
            h_index[nsp++] = (int)p;
        }
        st->last_time = t;
        ++st->seen;
    }
    *h_nspectra = nsp;
    *h_nblocks = nblocks;
    *h_timestamp = t;
    *h_gaps = gaps;
    return PV_OK;
}

extern "C" int pv_ab_unpack(const pv_ab_config* c, const void* d_chunk, long long bytes, const int* d_index,
                            long long nspectra, long long nblocks, float* d_out, void* stream) {
    PV_TRY(check_config(c, "ABDataAdapter"));
    if (bytes < 0 || nspectra < 0 || nblocks < 0 || nspectra > nblocks || (nblocks > 0 && !d_out) ||
        (nspectra > 0 && (!d_index || !d_chunk))) {
        pv::set_error("pv_ab_unpack: invalid arguments");
        return PV_ERR_ARG;
    }
    if (reinterpret_cast<uintptr_t>(d_chunk) % 8 != 0) {
        pv::set_error("pv_ab_unpack: the chunk must start on an 8-byte boundary");
        return PV_ERR_ARG;
    }
    const long long n = nblocks * c->channels;
    if (n == 0) return PV_OK;
    const long long npk = bytes / packet_bytes(c);
    const int grid = (int)std::min<long long>(pv::ceil_div<long long>(n, 256), 8LL * pv::sm_count());
    ab_unpack_kernel<<<grid, 256, 0, pv::as_stream(stream)>>>(reinterpret_cast<const uint2*>(d_chunk), npk,
                                                             c->channels, d_index, nspectra, nblocks, d_out);
    return pv::check_launch("ab_unpack_kernel");
}
