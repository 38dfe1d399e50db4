// ceos.cu -- RADARSAT-1 CEOS raw-data decode on sm_103a.
//
// Replaces the UBC MATLAB reader in code/data_process/CEOS (read_CEOS_raw.m,
// load_DATA_block.m, extract_AGC.m), which reads 8-line blocks with fread,
// cuts out the replica and decodes in the interpreter.  Here the caller's
// file bytes (the blocks that hold the wanted lines) are decoded on the
// device in one pass: four range cells per thread, 2-byte (I, Q) loads
// (every record offset is even), coalesced along a line.
//
// Layout (read_CEOS_raw.m:13-16,67-80): a file header, then blocks of
// lines_per_block lines of hpa = header + aux + 2 cells bytes, with a replica
// of `replica` bytes inside line replica_line of each block, right after its
// header and aux bytes.  Line k of a block therefore starts at k hpa, plus
// `replica` for k > replica_line - 1; its samples start at k hpa + header +
// aux, plus `replica` for k >= replica_line - 1.
// Decode (read_CEOS_raw.m:135-141): d = byte & 15, value 2 (d - 16 [d > 7]) + 1.
// AGC (extract_AGC.m:45-58): code = aux byte agc_byte & 63,
// dB = code - 24 [code > 31]; gain 1.5 10^(dB / 20) (load_DATA_block.m:58-69),
// taken from a 64-entry host table so device and host agree bit for bit.
#include "sarbp_internal.h"

namespace sarbp {
namespace {

constexpr int kCellsPerThread = 4;

__device__ __forceinline__ float ceos_value(unsigned d) {
    const int v = (int)(d & 15u);
    return (float)(2 * (v - 16 * (v > 7)) + 1);
}

__global__ void ceos_decode_kernel(const unsigned char *__restrict__ raw, CeosGeom g, const float *__restrict__ gains,
                                   float2 *__restrict__ echo, short *__restrict__ agc_db) {
    const int line = blockIdx.y;                       // 0-based within the request
    const int gl = g.first_line + line;                // line index in the file
    const int b = gl / g.lines_per_block, k = gl - b * g.lines_per_block;
    const long long base = (long long)b * g.block_bytes + (long long)k * g.line_bytes - g.raw_offset;
    const int r = g.replica_line - 1;
    const long long aux_off = base + g.header + g.agc_byte - 1 + (k > r ? g.replica : 0);
    const long long smp_off = base + g.header + g.aux + (k >= r ? g.replica : 0) + 2LL * g.first_cell;
    const unsigned code = raw[aux_off] & 63u;
    const float gain = g.apply_agc ? gains[code] : 1.f;
    if (agc_db && blockIdx.x == 0 && threadIdx.x == 0) agc_db[line] = (short)((int)code - 24 * (code > 31u));
    const unsigned short *s = reinterpret_cast<const unsigned short *>(raw + smp_off);
    float2 *dst = echo + (size_t)line * g.ncells;
    // kCellsPerThread cells per thread, strided by the block (coalesced), loads issued together
    const int step = blockDim.x;
    for (int c0 = blockIdx.x * step * kCellsPerThread + threadIdx.x; c0 < g.ncells;
         c0 += gridDim.x * step * kCellsPerThread) {
        unsigned iq[kCellsPerThread];
#pragma unroll
        for (int u = 0; u < kCellsPerThread; ++u) {
            const int c = c0 + u * step;
            iq[u] = c < g.ncells ? __ldg(&s[c]) : 0u;  // low byte I, high byte Q (file order)
        }
#pragma unroll
        for (int u = 0; u < kCellsPerThread; ++u) {
            const int c = c0 + u * step;
            if (c < g.ncells) dst[c] = make_float2(ceos_value(iq[u] & 255u) * gain, ceos_value(iq[u] >> 8) * gain);
        }
    }
}

}  // namespace

cudaError_t launch_ceos_decode(const unsigned char *raw, const CeosGeom &g, const float *gains, float2 *echo,
                               short *agc_db, cudaStream_t s) {
    if (g.nlines <= 0 || g.ncells <= 0) return cudaSuccess;
    const int threads = 256;
    const int bx = (g.ncells + threads * kCellsPerThread - 1) / (threads * kCellsPerThread);
    dim3 grid(bx < 8 ? bx : 8, g.nlines);
    ceos_decode_kernel<<<grid, threads, 0, s>>>(raw, g, gains, echo, agc_db);
    return cudaGetLastError();
}

}  // namespace sarbp
