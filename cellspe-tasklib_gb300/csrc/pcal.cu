// The PCal library on the GPU (include/cellspe_pcal.h): the reference's three
// multi-tone phase-cal extractors (spectrometer/src/IA-32/PhaseCal/PCal.cpp:
// 92-112 factory, 203-316 Trivial, 321-510 Shifting, 521-690 ImplicitShift)
// for sample pieces of any length and any sample offset.
//
// Fold: one thread per (bin, run of folding periods), so consecutive threads
// read consecutive samples; each sums its samples in registers (mixed down
// by the offset tone for Shifting, the oscillator phase kept as an exact
// integer residue (offset x n) mod fs) and adds its partial to the bin once.
// Tones: one block per picked DFT bin, the twiddle angle again an exact
// integer residue (bin x tone) mod N_bins.
#include "cellspe_gpu.h"
#include "cellspe_pcal.h"
#include "common.cuh"
#include "kernels.h"

#include <algorithm>
#include <cmath>
#include <vector>

struct cellspe_pcal {
    int kind = 0;
    uint64_t fs = 0, spacing = 0, offset = 0;
    int64_t nbins = 0, rotlen = 1;
    int ntones = 0;
    int64_t step = 0, first = 0;        // tone n is DFT bin first + n x step (Trivial: step 1)
    uint64_t pcal_index = 0, rot_index = 0;
    uint64_t samplecount = 0;
    bool finalized = false;
    float2* acc = nullptr;              // [nbins] bins (Trivial / ImplicitShift use .x)
    float2* tones = nullptr;            // [ntones] device result
    std::vector<float2> result;         // cached after the first cellspe_pcal_final
    int valid = 0;                      // tones whose bin is < nbins
    float* staging = nullptr;           // host input staged on the device
    cudaStream_t st = nullptr;
};

namespace {

constexpr int64_t PCAL_MAX_BINS = 1 << 28;
constexpr int64_t STAGE_FLOATS = 1 << 24;

uint64_t gcd_u64(uint64_t a, uint64_t b)
{
    while (b) {
        const uint64_t t = a % b;
        a = b;
        b = t;
    }
    return a;
}

// Thread g -> bin b = g % nbins, period run `part` = g / nbins.  Sample n of
// this piece lands in bin (pidx + n) % nbins, i.e. bin b holds samples
// n = n0(b) + p nbins.  MIX: x[n] exp(-2 pi i r / fs), r = offset (ridx + n) mod fs.
template <bool MIX>
__global__ void k_pcal_fold(const float* __restrict__ x, int64_t len, int64_t nbins, uint64_t pidx, int64_t per_part,
                            int64_t parts, uint64_t fs, uint64_t offset, uint64_t ridx, float2* __restrict__ acc)
{
    const int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (g >= nbins * parts) return;
    const int64_t b = g % nbins, part = g / nbins;
    const int64_t n0 = (int64_t)(((uint64_t)b + (uint64_t)nbins - pidx % (uint64_t)nbins) % (uint64_t)nbins);
    int64_t n = n0 + part * per_part * nbins;
    const int64_t nend = std::min<int64_t>(len, n0 + (part + 1) * per_part * nbins);
    if (n >= nend) return;
    float sr = 0.f, si = 0.f;
    if (MIX) {
        const float inv_fs = 1.0f / (float)fs;
        uint64_t r = (offset * ((ridx + (uint64_t)n) % fs)) % fs;
        const uint64_t dr = (offset * ((uint64_t)nbins % fs)) % fs;
        for (; n < nend; n += nbins) {
            float sn, cs;
            sincospif(-2.0f * ((float)r * inv_fs), &sn, &cs);
            const float v = __ldg(x + n);
            sr = fmaf(v, cs, sr);
            si = fmaf(v, sn, si);
            r += dr;
            if (r >= fs) r -= fs;
        }
        atomicAdd(&acc[b].x, sr);
        atomicAdd(&acc[b].y, si);
    } else {
        for (; n < nend; n += nbins) sr += __ldg(x + n);
        atomicAdd(&acc[b].x, sr);
    }
}

// out[t] = (1 / nbins) sum_b acc[b] exp(-2 pi i bin_t b / nbins), bin_t = first + t step
__global__ void k_pcal_tones(const float2* __restrict__ acc, int64_t nbins, int64_t first, int64_t step, bool real,
                             float2* __restrict__ out)
{
    const int t = blockIdx.x;
    const uint64_t k = (uint64_t)(first + (int64_t)t * step);
    const float inv = 1.0f / (float)nbins;
    float re = 0.f, im = 0.f;
    for (int64_t b = threadIdx.x; b < nbins; b += blockDim.x) {
        const uint64_t m = (k * (uint64_t)b) % (uint64_t)nbins;
        float sn, cs;
        sincospif(-2.0f * ((float)m * inv), &sn, &cs);
        const float2 a = acc[b];
        const float ai = real ? 0.f : a.y;
        re += a.x * cs - ai * sn;
        im += a.x * sn + ai * cs;
    }
    __shared__ float sre[32], sim[32];
    for (int o = 16; o > 0; o >>= 1) {
        re += __shfl_xor_sync(0xffffffffu, re, o);
        im += __shfl_xor_sync(0xffffffffu, im, o);
    }
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) {
        sre[w] = re;
        sim[w] = im;
    }
    __syncthreads();
    if (w == 0) {
        const int nw = blockDim.x >> 5;
        re = l < nw ? sre[l] : 0.f;
        im = l < nw ? sim[l] : 0.f;
        for (int o = 16; o > 0; o >>= 1) {
            re += __shfl_xor_sync(0xffffffffu, re, o);
            im += __shfl_xor_sync(0xffffffffu, im, o);
        }
        if (l == 0) out[t] = make_float2(re * inv, im * inv);
    }
}

int pc_err(int code, const char* msg) { return cs_set_error(code, msg); }
int pc_cuda(cudaError_t e) { return cs_set_error(CELLSPE_ERR_CUDA, cudaGetErrorString(e)); }

int fold_piece(cellspe_pcal* pc, const float* d_x, int64_t len)
{
    const bool mix = pc->kind == CELLSPE_PCAL_SHIFTING;
    const int64_t periods = (len + pc->nbins - 1) / pc->nbins + 1;
    // enough (bin, run) threads to fill the GPU, at least one period per run
    const int64_t want = std::max<int64_t>(1, (int64_t)152 * 2048 / std::max<int64_t>(1, std::min<int64_t>(pc->nbins, 152 * 2048)));
    const int64_t parts = std::max<int64_t>(1, std::min<int64_t>(periods, want));
    const int64_t per_part = (periods + parts - 1) / parts;
    const int64_t threads = pc->nbins * parts;
    const int64_t blocks = (threads + 255) / 256;
    if (blocks > 0x7fffffffLL) return pc_err(CELLSPE_ERR_UNSUPPORTED, "pcal_extract: piece too long for one launch");
    if (mix)
        k_pcal_fold<true><<<(unsigned)blocks, 256, 0, pc->st>>>(d_x, len, pc->nbins, pc->pcal_index, per_part, parts,
                                                                pc->fs, pc->offset, pc->rot_index, pc->acc);
    else
        k_pcal_fold<false><<<(unsigned)blocks, 256, 0, pc->st>>>(d_x, len, pc->nbins, pc->pcal_index, per_part, parts,
                                                                 pc->fs, pc->offset, pc->rot_index, pc->acc);
    cs_count_launches(1);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return pc_cuda(e);
    pc->pcal_index = (pc->pcal_index + (uint64_t)len) % (uint64_t)pc->nbins;
    pc->rot_index = (pc->rot_index + (uint64_t)len) % (uint64_t)pc->rotlen;
    pc->samplecount += (uint64_t)len;
    return 0;
}

}  // namespace

extern "C" {

cellspe_pcal* cellspe_pcal_new(double bandwidth_hz, double pcal_spacing_hz, int pcal_offset_hz,
                               unsigned long long sampleoffset)
{
    const double fsd = 2.0 * bandwidth_hz;
    if (!(bandwidth_hz > 0) || !(pcal_spacing_hz > 0) || pcal_offset_hz < 0 || fsd != std::floor(fsd) ||
        pcal_spacing_hz != std::floor(pcal_spacing_hz) || fsd >= 4294967296.0) {
        cs_set_error(CELLSPE_ERR_ARG, "pcal_new: bandwidth and spacing must be positive whole numbers of Hz "
                                      "(2 x bandwidth < 2^32), offset >= 0");
        return nullptr;
    }
    auto* pc = new cellspe_pcal();
    pc->fs = (uint64_t)fsd;
    pc->spacing = (uint64_t)pcal_spacing_hz;
    pc->offset = (uint64_t)pcal_offset_hz;
    const int64_t Np = (int64_t)(pc->fs / gcd_u64(pc->spacing, pc->fs));
    if (pc->offset == 0) {                                       // PCal.cpp:99-101
        pc->kind = CELLSPE_PCAL_TRIVIAL;
        pc->nbins = Np;
        pc->ntones = (int)std::floor(bandwidth_hz / pcal_spacing_hz);
        pc->step = 1;
        pc->first = 0;
    } else {
        const int64_t No = (int64_t)(pc->fs / gcd_u64(pc->offset, pc->fs));
        pc->ntones = (int)std::floor((bandwidth_hz - pcal_offset_hz) / pcal_spacing_hz) + 1;
        if (No % Np == 0) {                                      // PCal.cpp:106-108
            pc->kind = CELLSPE_PCAL_IMPLICIT_SHIFT;
            pc->nbins = No;
            pc->first = (int64_t)std::floor((double)No * (double)pc->offset / fsd);
        } else {
            pc->kind = CELLSPE_PCAL_SHIFTING;
            pc->nbins = Np;
            pc->rotlen = No;
            pc->first = 0;
        }
        pc->step = (int64_t)std::floor((double)pc->nbins * (pcal_spacing_hz / fsd));
    }
    if (pc->nbins > PCAL_MAX_BINS || pc->ntones < 0) {
        cs_set_error(CELLSPE_ERR_UNSUPPORTED, "pcal_new: more than 2^28 folding bins");
        delete pc;
        return nullptr;
    }
    pc->valid = 0;
    for (int t = 0; t < pc->ntones; t++)
        if (pc->first + (int64_t)t * pc->step < pc->nbins) pc->valid = t + 1;
        else break;
    cudaError_t e = cudaStreamCreate(&pc->st);                   // ordered after the legacy default stream
    if (e == cudaSuccess) e = cudaMalloc(&pc->acc, (size_t)pc->nbins * sizeof(float2));
    if (e == cudaSuccess) e = cudaMalloc(&pc->tones, (size_t)std::max(1, pc->ntones) * sizeof(float2));
    if (e != cudaSuccess) {
        pc_cuda(e);
        cellspe_pcal_free(pc);
        return nullptr;
    }
    if (cellspe_pcal_clear(pc) || cellspe_pcal_adjust_sample_offset(pc, sampleoffset)) {
        cellspe_pcal_free(pc);
        return nullptr;
    }
    return pc;
}

void cellspe_pcal_free(cellspe_pcal* pc)
{
    if (!pc) return;
    if (pc->st) cudaStreamSynchronize(pc->st);
    cudaFree(pc->acc);
    cudaFree(pc->tones);
    cudaFree(pc->staging);
    if (pc->st) cudaStreamDestroy(pc->st);
    delete pc;
}

int cellspe_pcal_kind(const cellspe_pcal* pc) { return pc ? pc->kind : -CELLSPE_ERR_ARG; }
int cellspe_pcal_length(const cellspe_pcal* pc) { return pc ? pc->ntones : -CELLSPE_ERR_ARG; }
long long cellspe_pcal_nbins(const cellspe_pcal* pc) { return pc ? pc->nbins : -CELLSPE_ERR_ARG; }
double cellspe_pcal_seconds(const cellspe_pcal* pc) { return pc && pc->fs ? (double)pc->samplecount / (double)pc->fs : 0.0; }

int cellspe_pcal_clear(cellspe_pcal* pc)
{
    if (!pc) return pc_err(CELLSPE_ERR_ARG, "pcal_clear: null extractor");
    pc->samplecount = 0;
    pc->finalized = false;
    pc->result.clear();
    cudaError_t e = cudaMemsetAsync(pc->acc, 0, (size_t)pc->nbins * sizeof(float2), pc->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(pc->st);
    return e == cudaSuccess ? 0 : pc_cuda(e);
}

int cellspe_pcal_adjust_sample_offset(cellspe_pcal* pc, unsigned long long sampleoffset)
{
    if (!pc) return pc_err(CELLSPE_ERR_ARG, "pcal_adjust_sample_offset: null extractor");
    pc->pcal_index = sampleoffset % (uint64_t)pc->nbins;
    pc->rot_index = sampleoffset % (uint64_t)pc->rotlen;
    return 0;
}

int cellspe_pcal_extract(cellspe_pcal* pc, const float* samples, long long len, int memory)
{
    if (!pc || len < 0 || (len > 0 && !samples)) return pc_err(CELLSPE_ERR_ARG, "pcal_extract: bad arguments");
    if (pc->finalized) return pc_err(CELLSPE_ERR_ARG, "pcal_extract: extractor finalised; clear it first");
    if (len == 0) return 0;
    if (memory == CELLSPE_MEM_DEVICE) {
        int rc = fold_piece(pc, samples, len);
        if (rc) return rc;
    } else {
        if (!pc->staging) {
            const cudaError_t e = cudaMalloc(&pc->staging, (size_t)STAGE_FLOATS * sizeof(float));
            if (e != cudaSuccess) return pc_cuda(e);
        }
        for (long long o = 0; o < len; o += STAGE_FLOATS) {
            const int64_t n = std::min<int64_t>(STAGE_FLOATS, len - o);
            cudaError_t e = cudaMemcpyAsync(pc->staging, samples + o, (size_t)n * sizeof(float), cudaMemcpyHostToDevice,
                                            pc->st);
            if (e != cudaSuccess) return pc_cuda(e);
            int rc = fold_piece(pc, pc->staging, n);
            if (rc) return rc;
            e = cudaStreamSynchronize(pc->st);                 // staging reused by the next piece
            if (e != cudaSuccess) return pc_cuda(e);
        }
    }
    const cudaError_t e = cudaStreamSynchronize(pc->st);
    return e == cudaSuccess ? 0 : pc_cuda(e);
}

long long cellspe_pcal_final(cellspe_pcal* pc, void* out)
{
    if (!pc || (!out && pc->ntones > 0)) return -pc_err(CELLSPE_ERR_ARG, "pcal_final: bad arguments");
    if (!pc->finalized) {
        if (pc->valid > 0) {
            const bool real = pc->kind != CELLSPE_PCAL_SHIFTING;
            k_pcal_tones<<<pc->valid, 256, 0, pc->st>>>(pc->acc, pc->nbins, pc->first, pc->step, real, pc->tones);
            cs_count_launches(1);
            cudaError_t e = cudaGetLastError();
            pc->result.assign(pc->valid, make_float2(0.f, 0.f));
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(pc->result.data(), pc->tones, (size_t)pc->valid * sizeof(float2),
                                    cudaMemcpyDeviceToHost, pc->st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(pc->st);
            if (e != cudaSuccess) return -pc_cuda(e);
        }
        pc->finalized = true;
    }
    if (pc->valid > 0) std::copy(pc->result.begin(), pc->result.end(), static_cast<float2*>(out));
    return (long long)pc->samplecount;
}

}  // extern "C"
