"""cellspe_spectrometer_noalloc, the entry point that allocates no device memory.

It serves callers that cannot call cudaMalloc while they run (real-time loops
that must not stall on the allocator, work issued during CUDA graph capture,
hosts with a fixed device footprint).  The test calls it through the C ABI
twice in a row and checks each result against the allocating entry point
cellspe_spectrometer on the same device buffers, plus the rejection of a job
larger than the static scratch and of arguments the allocating entry point
rejects too.

Tolerance: both entry points run the same kernels, but this one builds its
FFT twiddle, window and phase-cal rotator tables on the device with the
device's FP64 cos/sin, while cellspe_spectrometer builds them on the host with
the C library's; the two may differ in the last bit of a double, which can move
an FP32-rounded table entry by one ulp, and a job regrouped to fit the static
scratch sums its partial spectra in a different order.  Results are therefore
compared at the spectrometer tests' relative tolerance (1e-5), not bit for bit.

This file is collected last so that a failure here never hides another test.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _run_pair(cg, torch, raw, N, overlap, window, K, nspec, nsub, levels, pcal, rotlen=32, offset=0.0, calls=2):
    """Allocating result once, then `calls` no-alloc calls compared with it."""
    kw = dict(layout=cg.SPEC_PLANES, levels=levels)
    if pcal:
        kw.update(tonebins=32, rotatorlen=rotlen, ntones=16, offset_hz=offset, fs_hz=32e6)
    shape = (nsub, nspec, N // 2 + 1)
    ref = torch.zeros(shape, dtype=torch.float32, device="cuda")
    ref_bins = torch.zeros((nsub, nspec, 32), dtype=torch.complex64, device="cuda") if pcal else None
    ref_tones = torch.zeros((nsub, nspec, 16), dtype=torch.complex64, device="cuda") if pcal else None
    cg.spectrometer(cg.spec_params(N, overlap, window, K, nspec, nsub, raw.numel(), **kw), raw, ref, ref_bins,
                    ref_tones)
    torch.cuda.synchronize()
    ref_np = ref.cpu().numpy()
    for call in range(calls):
        out = torch.full(shape, float("nan"), dtype=torch.float32, device="cuda")
        bins = torch.full_like(ref_bins, float("nan")) if pcal else None
        tones = torch.full_like(ref_tones, float("nan")) if pcal else None
        stream = torch.cuda.current_stream().cuda_stream
        cg.spectrometer_noalloc(cg.spec_params(N, overlap, window, K, nspec, nsub, raw.numel(), **kw), raw, out,
                                bins, tones, stream=stream)
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert np.isfinite(got).all(), f"call {call}: unwritten output"
        assert _rel(got, ref_np) < TOL, f"call {call}"
        if pcal:
            assert _rel(bins.cpu().numpy(), ref_bins.cpu().numpy()) < TOL
            assert _rel(tones.cpu().numpy(), ref_tones.cpu().numpy()) < TOL


def _planes(torch, nsub, nbytes, seed):
    g = torch.Generator(device="cuda").manual_seed(seed)
    return torch.randint(0, 256, (nsub * nbytes,), dtype=torch.uint8, device="cuda", generator=g)


@pytest.mark.parametrize("nsub,N,overlap,K,nspec,pcal,levels", [
    (4, 4096, 2, 16, 2, True, "LEVELS_MARK5B"),     # default chunking, phase-cal on
    (16, 65536, 2, 512, 1, False, "LEVELS_MARK5B"), # the 16-subband 65536-point shape: chunks regrouped to fit
    (8, 8192, 1, 32, 2, True, "LEVELS_VDIF"),       # deframed VDIF planes with the VDIF level table
])
def test_noalloc_matches_allocating_entry_point(cg, nsub, N, overlap, K, nspec, pcal, levels):
    import torch

    raw = _planes(torch, nsub, N * K * nspec // 4, nsub * 1000 + N)
    _run_pair(cg, torch, raw, N, overlap, 2, K, nspec, nsub, getattr(cg, levels), pcal)


def test_noalloc_shapes_in_sequence(cg):
    """Consecutive calls on one stream that change N, window, rotator length and
    chunking rebuild the tables and scratch each time: the first shape again at
    the end gives its result again."""
    import torch

    shapes = [
        # nsub, N, overlap, window, K, nspec, rotlen, offset (Hz)
        (16, 65536, 2, 2, 512, 1, 32, 0.0),     # regrouped chunks, phase-cal
        (4, 4096, 1, 1, 64, 3, 1024, 31250.0), # cosine window, 31.25 kHz offset: a 1024-sample rotator
        (1, 1024, 2, 0, 8, 4, 32, 0.0),         # no window, one subband
        (16, 65536, 2, 2, 512, 1, 32, 0.0),     # the first shape again
    ]
    for i, (nsub, N, ovl, win, K, nspec, rotlen, off) in enumerate(shapes):
        raw = _planes(torch, nsub, N * K * nspec // 4, 77 + (i % 3))
        _run_pair(cg, torch, raw, N, ovl, win, K, nspec, nsub, cg.LEVELS_MARK5B, True, rotlen=rotlen, offset=off,
                  calls=1)


def test_noalloc_rejects_jobs_beyond_the_scratch_maximum(cg):
    import torch

    nsub, N, K, nspec = 16, 65536, 1, 8            # 128 rows x 32769 bins > 4,194,304 floats
    raw = torch.zeros((nsub * N * K * nspec // 4,), dtype=torch.uint8, device="cuda")
    out = torch.zeros((nsub, nspec, N // 2 + 1), dtype=torch.float32, device="cuda")
    p = cg.spec_params(N, 1, 0, K, nspec, nsub, raw.numel(), layout=cg.SPEC_PLANES)
    with pytest.raises(cg.CellspeError) as e:
        cg.spectrometer_noalloc(p, raw, out)
    assert e.value.code == cg.ERR_ARG and "scratch maximum" in str(e.value)


def test_noalloc_rejects_what_the_allocating_entry_point_rejects(cg):
    """The same argument checks: an unknown input layout and phase-cal without a
    sample rate fail in both entry points with CELLSPE_ERR_ARG."""
    import torch

    N, K = 4096, 4
    raw = torch.zeros((N * K // 4,), dtype=torch.uint8, device="cuda")
    out = torch.zeros((1, 1, N // 2 + 1), dtype=torch.float32, device="cuda")
    bins = torch.zeros((1, 1, 32), dtype=torch.complex64, device="cuda")
    bad_layout = cg.spec_params(N, 1, 0, K, 1, 1, raw.numel(), layout=7)
    no_fs = cg.spec_params(N, 1, 0, K, 1, 1, raw.numel(), layout=cg.SPEC_PLANES, tonebins=32, rotatorlen=32)
    for p, b in ((bad_layout, None), (no_fs, bins)):
        for fn in (cg.spectrometer, cg.spectrometer_noalloc):
            with pytest.raises(cg.CellspeError) as e:
                fn(p, raw, out, b)
            assert e.value.code == cg.ERR_ARG
