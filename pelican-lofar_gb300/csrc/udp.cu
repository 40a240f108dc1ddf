// LOFAR UDP ingest: chunks of station packets -> TimeSeriesDataSetC32.
//
// Replaces AdapterTimeSeriesDataSet::deserialise/_readData
// (lib/src/AdapterTimeSeriesDataSet.cpp:78-293).  The reference copies each
// packet through a temporary buffer and scatters it element by element on
// one host thread; here the chunk of packets is one device buffer (copied in
// once) and the scatter is a byte transpose on the GPU.
//
// A packet is a 16-byte header (lib/LofarUdpHeader.h:25-35), then the data,
// subband-major: for each subband, each time, each polarisation one complex
// int8 or int16 (AdapterTimeSeriesDataSet.cpp:229-288), then, for fixed-size
// packets, padding up to sizeof(UDPPacket) = 8148 bytes.  Time t of packet k
// is sample k*spp + t of the series [subband][pol], and a series is
// contiguous in time in TimeSeriesDataSetC32 (lib/TimeSeriesDataSet.h:145-151).
//
// The kernel is HBM-bound: per element it reads 2 or 4 bytes and writes 4
// (int16 output) or 8 (complex float).  A CTA row is one subband's
// spp*npol elements of a packet; its threads read consecutive elements of
// the packet (coalesced) and each polarisation's threads write spp
// consecutive samples of their series.  A CTA walks several packets, so a
// series row grows by spp samples per packet.
#include <algorithm>
#include <cstring>

#include "pv_internal.cuh"

namespace {

constexpr int kHeaderBytes = 16;
constexpr long long kFixedPacketBytes = 8148;  // sizeof(UDPPacket): 16 + 8130, 4-byte aligned
constexpr long long kFixedDataBytes = 8130;

template <int BITS, bool C32>
__global__ void __launch_bounds__(256)
udp_unpack_kernel(const unsigned char* __restrict__ chunk, long long packet_bytes, int npackets,
                  int nsub, int npol, int spp, int packets_per_cta, void* __restrict__ out) {
    const int x = threadIdx.x;  // t * npol + p
    const int s = blockIdx.y * blockDim.y + threadIdx.y;
    if (s >= nsub) return;
    const int t = x / npol, p = x - t * npol;
    const long long nt = (long long)npackets * spp;
    const int k0 = blockIdx.x * packets_per_cta;
    const int k1 = min(npackets, k0 + packets_per_cta);
    constexpr int EB = BITS / 4;  // bytes of one complex element
    const unsigned char* src = chunk + kHeaderBytes + (long long)((s * spp + t) * npol + p) * EB;
    const long long row = ((long long)s * npol + p) * nt + t;
#pragma unroll 4
    for (int k = k0; k < k1; ++k) {
        const unsigned char* q = src + (long long)k * packet_bytes;
        int re, im;
        if (BITS == 16) {
            const short2 v = __ldg(reinterpret_cast<const short2*>(q));
            re = v.x;
            im = v.y;
        } else {
            const char2 v = __ldg(reinterpret_cast<const char2*>(q));
            re = v.x;
            im = v.y;
        }
        const long long o = row + (long long)k * spp;
        if (C32)
            __stcs(reinterpret_cast<float2*>(out) + o, make_float2((float)re, (float)im));
        else
            reinterpret_cast<short2*>(out)[o] = make_short2((short)re, (short)im);
    }
}

int check_config(const pv_udp_config* c) {
    if (!c) {
        pv::set_error("pv_udp: null config");
        return PV_ERR_ARG;
    }
    if (c->sample_bits != 8 && c->sample_bits != 16) {
        pv::set_error("AdapterTimeSeriesDataSet: Sample size (%d bits) not supported.", c->sample_bits);
        return PV_ERR_CONFIG;
    }
    if (c->packets_per_chunk <= 0 || c->samples_per_packet <= 0 || c->nchan <= 0 || c->nsub <= 0 ||
        c->npol <= 0) {
        pv::set_error("AdapterTimeSeriesDataSet: packets, samples, channels, subbands and "
                      "polarisations must be positive");
        return PV_ERR_CONFIG;
    }
    if (c->sample_bits == 16 && c->npol != 2) {
        pv::set_error("AdapterTimeSeriesDataSet: 16-bit packets carry two polarisations");
        return PV_ERR_CONFIG;
    }
    if ((long long)c->samples_per_packet * c->npol > 256) {  // one CTA row per packet subband
        pv::set_error("AdapterTimeSeriesDataSet: samplesPerPacket x nRawPolarisations above 256");
        return PV_ERR_CONFIG;
    }
    return PV_OK;
}

}  // namespace

extern "C" int pv_udp_check(const pv_udp_config* c, long long chunk_bytes, long long* h_packet_bytes,
                            int* h_nblocks) {
    PV_TRY(check_config(c));
    const long long samples = (long long)c->nsub * c->npol * c->samples_per_packet;
    const long long useful_bits = samples * c->sample_bits * 2;  // complex
    const long long psize = c->fixed_size_packets ? kFixedPacketBytes : kHeaderBytes + useful_bits / 8;
    const long long udp_bits = c->fixed_size_packets ? kFixedDataBytes * 8 : useful_bits;
    if (chunk_bytes != psize * c->packets_per_chunk) {
        pv::set_error("AdapterTimeSeriesDataSet: Chunk size '%lld' != '%lld' expected for %d UDP packets.",
                      chunk_bytes, psize * c->packets_per_chunk, c->packets_per_chunk);
        return PV_ERR_CONFIG;
    }
    if (useful_bits > udp_bits) {
        pv::set_error("AdapterTimeSeriesDataSet: Dimensions decribe more data than fits into a UDP "
                      "packet!  (%lld > %lld",
                      useful_bits, udp_bits);
        return PV_ERR_CONFIG;
    }
    const long long times = (long long)c->samples_per_packet * c->packets_per_chunk;
    if (times % c->nchan != 0) {
        pv::set_error("AdapterTimeSeriesDataSet: Number of time samples must be evenly divisible by "
                      "the number of samples in a block.");
        return PV_ERR_CONFIG;
    }
    if (h_packet_bytes) *h_packet_bytes = psize;
    if (h_nblocks) *h_nblocks = (int)(times / c->nchan);
    return PV_OK;
}

extern "C" int pv_udp_unpack(const pv_udp_config* c, const void* d_chunk, long long chunk_bytes,
                             void* d_out, int out_type, void* stream) {
    long long psize = 0;
    int nblocks = 0;
    PV_TRY(pv_udp_check(c, chunk_bytes, &psize, &nblocks));
    if (!d_chunk || !d_out || (out_type != PV_UDP_OUT_C32 && out_type != PV_UDP_OUT_I16)) {
        pv::set_error("pv_udp_unpack: invalid arguments");
        return PV_ERR_ARG;
    }
    const uintptr_t align = c->sample_bits == 16 ? 4 : 2;
    if (reinterpret_cast<uintptr_t>(d_chunk) % align != 0 ||
        reinterpret_cast<uintptr_t>(d_out) % (out_type == PV_UDP_OUT_C32 ? 8 : 4) != 0) {
        pv::set_error("pv_udp_unpack: chunk or output pointer not aligned to its element");
        return PV_ERR_ARG;
    }
    const int bx = c->samples_per_packet * c->npol;
    const int by = std::max(1, 256 / bx);
    constexpr int kPacketsPerCta = 8;
    const dim3 grid((unsigned)pv::ceil_div(c->packets_per_chunk, kPacketsPerCta),
                    (unsigned)pv::ceil_div(c->nsub, by));
    if (grid.y > 65535u) {
        pv::set_error("pv_udp_unpack: too many subbands");
        return PV_ERR_ARG;
    }
    const dim3 block((unsigned)bx, (unsigned)by);
    auto* in = reinterpret_cast<const unsigned char*>(d_chunk);
    cudaStream_t s = pv::as_stream(stream);
    const bool c32 = out_type == PV_UDP_OUT_C32;
    if (c->sample_bits == 16) {
        if (c32)
            udp_unpack_kernel<16, true><<<grid, block, 0, s>>>(in, psize, c->packets_per_chunk, c->nsub,
                                                              c->npol, c->samples_per_packet,
                                                              kPacketsPerCta, d_out);
        else
            udp_unpack_kernel<16, false><<<grid, block, 0, s>>>(in, psize, c->packets_per_chunk, c->nsub,
                                                               c->npol, c->samples_per_packet,
                                                               kPacketsPerCta, d_out);
    } else {
        if (c32)
            udp_unpack_kernel<8, true><<<grid, block, 0, s>>>(in, psize, c->packets_per_chunk, c->nsub,
                                                             c->npol, c->samples_per_packet,
                                                             kPacketsPerCta, d_out);
        else
            udp_unpack_kernel<8, false><<<grid, block, 0, s>>>(in, psize, c->packets_per_chunk, c->nsub,
                                                              c->npol, c->samples_per_packet,
                                                              kPacketsPerCta, d_out);
    }
    return pv::check_launch("udp_unpack_kernel");
}

extern "C" int pv_udp_time(const pv_udp_config* c, const void* h_packet, double* h_timestamp,
                           double* h_block_rate) {
    if (!c || !h_packet || !h_timestamp || !h_block_rate) {
        pv::set_error("pv_udp_time: invalid arguments");
        return PV_ERR_ARG;
    }
    uint32_t ts, seq;
    std::memcpy(&ts, static_cast<const unsigned char*>(h_packet) + 8, 4);
    std::memcpy(&seq, static_cast<const unsigned char*>(h_packet) + 12, 4);
    const unsigned tot = c->clock_mhz == 160 ? 156250u : (ts % 2 == 0 ? 195313u : 195312u);
    *h_timestamp = ts + (1.0 * seq) / tot;
    *h_block_rate = 1.0 / tot;
    return PV_OK;
}
