// minicorrelator_gpu -- the minicorrelator entry point on the GB300 engine.
//
// Usage: minicorrelator_gpu [-h] [stations] [integrations]
//
// Mirrors the reference's minicorrelator (minicorrelator/minicorrelator_ppu.c,
// minicorrelator.h:84-119): 6 stations of 2-bit data, a 1024-point FFT, the
// PPU's deterministic raw pattern (17*i + 3*j) % 256 for station i, byte j
// (minicorrelator_ppu.c:131-133), 256 x 16 KiB of raw data per station and
// integration over all FFTs, autocorrelations plus the 15 baselines.  It
// prints the data volume, the achieved raw-input rate in Gbit/s (like
// minicorrelator_ppu.c:207-231) and the first four values of every product
// (:242-251).  The reference's SPU kernels are placeholders (dummy LUT, FFT
// compiled out, see minicorrelator_spu.c:314-317, :342-348); here each
// station's bytes are offset-binary 2-bit samples through the full path:
// unpack -> real FFT -> conjugate cross-multiply-accumulate (FP32).
// Products are written as planar [Re x C][Im x C] blocks, the layout of
// the reference's autocorrelation / baseline result buffers.
#include "../../../include/cellspe_gpu.h"

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

int main(int argc, char** argv)
{
    if (argc > 1 && !strcmp(argv[1], "-h")) {
        printf("Usage: %s [-h] [stations=6] [integrations=1]\n"
               "  Correlates the reference minicorrelator's synthetic pattern on the GPU.\n", argv[0]);
        return 0;
    }
    const int S = argc > 1 ? atoi(argv[1]) : 6;
    const int nint = argc > 2 ? atoi(argv[2]) : 1;
    const int N = 1024, C = N / 2;
    const long long raw_bytes = 256LL * 16384;                 // PPU_RAW_1SPEBYTES
    const int K = (int)(raw_bytes * 4 / N / nint);              // FFTs per integration
    const int P = S * (S + 1) / 2;
    if (S < 2 || K < 1) { fprintf(stderr, "bad arguments\n"); return 1; }
    printf("\nUsing %d stations on the GPU.\nDataset: %lld kB raw data per station, %d FFTs of %d points per integration, "
           "%d integrations, %d baselines\n", S, raw_bytes / 1024, K, N, nint, S * (S - 1) / 2);

    unsigned char* raw = (unsigned char*)cellspe_host_alloc((size_t)S * raw_bytes);
    float* vis = (float*)cellspe_host_alloc((size_t)P * C * 8);
    if (!raw || !vis) { fprintf(stderr, "%s\n", cellspe_last_error()); return 1; }
    for (int i = 0; i < S; i++)
        for (long long j = 0; j < raw_bytes; j++) raw[(size_t)i * raw_bytes + j] = (unsigned char)((17 * i + 3 * j) % 256);

    cellspe_fx_params p;
    memset(&p, 0, sizeof p);
    p.n_inputs = S; p.fft_points = N; p.n_segments = K; p.x_mode = CELLSPE_X_FP32;
    p.vis_order = CELLSPE_VIS_BASELINE_MAJOR; p.levels = CELLSPE_LEVELS_OFFSET_BINARY;
    p.bytes_per_input = raw_bytes; p.memory = CELLSPE_MEM_HOST;
    std::vector<float> planar((size_t)P * 2 * C);
    double total_s = 0;
    int rc = 0;
    for (int it = 0; it < nint && !rc; it++) {
        p.start_sample = (long long)it * K * N;
        auto t0 = std::chrono::steady_clock::now();
        rc = cellspe_fx_correlate(&p, raw, nullptr, vis);
        total_s += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        for (int q = 0; q < P; q++)
            for (int c = 0; c < C; c++) {
                planar[(size_t)q * 2 * C + c] = vis[((size_t)q * C + c) * 2];
                planar[(size_t)q * 2 * C + C + c] = vis[((size_t)q * C + c) * 2 + 1];
            }
    }
    if (rc) { fprintf(stderr, "correlation failed: %s\n", cellspe_last_error()); return 1; }
    const double gbit = (double)S * raw_bytes * 8 / 1e9;
    printf("Total time %.6f s for %.3f Gbit of raw data: %.3f Gbit/s aggregate\n", total_s, gbit, gbit / total_s);
    for (int i = 0; i < S; i++)
        for (int j = 0; j <= i; j++) {
            const float* b = planar.data() + (size_t)(i * (i + 1) / 2 + j) * 2 * C;
            printf("%s %d-%d : re {%g %g %g %g} im {%g %g %g %g}\n", i == j ? "auto    " : "baseline", i, j,
                   b[0], b[1], b[2], b[3], b[C], b[C + 1], b[C + 2], b[C + 3]);
        }
    cellspe_host_free(raw);
    cellspe_host_free(vis);
    return 0;
}
