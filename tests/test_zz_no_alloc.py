"""cellspe_spectrometer_noalloc, the entry point that allocates no device memory.

It serves callers that cannot call cudaMalloc while they run (real-time loops
that must not stall on the allocator, work issued during CUDA graph capture,
hosts with a fixed device footprint).  The test calls it through the C ABI
twice in a row and checks each result against the allocating entry point
cellspe_spectrometer on the same device buffers, at the spectrometer tests'
tolerance, plus the rejection of a job larger than the static scratch.
This file is collected last so that a failure here never hides another test.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("nsub,N,overlap,K,nspec,pcal", [
    (4, 4096, 2, 16, 2, True),      # default chunking, phase-cal on
    (16, 65536, 2, 512, 1, False),  # the 16-subband 65536-point shape: chunks regrouped to fit
])
def test_noalloc_matches_allocating_entry_point(cg, nsub, N, overlap, K, nspec, pcal):
    import torch

    bytes_per_sub = N * K * nspec // 4
    g = torch.Generator(device="cuda").manual_seed(nsub * 1000 + N)
    raw = torch.randint(0, 256, (nsub * bytes_per_sub,), dtype=torch.uint8, device="cuda", generator=g)
    kw = dict(layout=cg.SPEC_PLANES, levels=cg.LEVELS_MARK5B)
    if pcal:
        kw.update(tonebins=32, rotatorlen=32, ntones=16, offset_hz=0.0, fs_hz=32e6)
    shape = (nsub, nspec, N // 2 + 1)
    ref = torch.zeros(shape, dtype=torch.float32, device="cuda")
    ref_bins = torch.zeros((nsub, nspec, 32), dtype=torch.complex64, device="cuda") if pcal else None
    ref_tones = torch.zeros((nsub, nspec, 16), dtype=torch.complex64, device="cuda") if pcal else None
    cg.spectrometer(cg.spec_params(N, overlap, 2, K, nspec, nsub, raw.numel(), **kw), raw, ref, ref_bins, ref_tones)
    torch.cuda.synchronize()
    ref_np = ref.cpu().numpy()
    for call in range(2):
        out = torch.full(shape, float("nan"), dtype=torch.float32, device="cuda")
        bins = torch.zeros_like(ref_bins) if pcal else None
        tones = torch.zeros_like(ref_tones) if pcal else None
        stream = torch.cuda.current_stream().cuda_stream
        cg.spectrometer_noalloc(cg.spec_params(N, overlap, 2, K, nspec, nsub, raw.numel(), **kw), raw, out,
                                bins, tones, stream=stream)
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert np.isfinite(got).all(), f"call {call}: unwritten output"
        assert _rel(got, ref_np) < TOL, f"call {call}"
        if pcal:
            assert _rel(bins.cpu().numpy(), ref_bins.cpu().numpy()) < TOL
            assert _rel(tones.cpu().numpy(), ref_tones.cpu().numpy()) < TOL


def test_noalloc_rejects_jobs_beyond_the_scratch_maximum(cg):
    import torch

    nsub, N, K, nspec = 16, 65536, 1, 8            # 128 rows x 32769 bins > 4,194,304 floats
    raw = torch.zeros((nsub * N * K * nspec // 4,), dtype=torch.uint8, device="cuda")
    out = torch.zeros((nsub, nspec, N // 2 + 1), dtype=torch.float32, device="cuda")
    p = cg.spec_params(N, 1, 0, K, nspec, nsub, raw.numel(), layout=cg.SPEC_PLANES)
    with pytest.raises(cg.CellspeError) as e:
        cg.spectrometer_noalloc(p, raw, out)
    assert e.value.code == cg.ERR_ARG and "scratch maximum" in str(e.value)
