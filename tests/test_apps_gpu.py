"""Entry-point programs: swspectrometer_gpu and minicorrelator_gpu (run as processes)."""
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
PKG = Path(__file__).resolve().parent.parent / "cellspe-tasklib_gb300"


def test_swspectrometer_cli_matches_oracle(cg, orc, tmp_path):
    import synth

    N, K, fs, nspec, ch = 4096, 8, 32e6, 2, 3
    words, _ = synth.mark5b_subbands(16, N * K * nspec, fs_hz=fs, seed=31, n_channels=N // 2, pcal_amp=0.2)
    data = tmp_path / "scan.m5b"
    words.tofile(data)
    ini = tmp_path / "spec.ini"
    ini.write_text(f"""[Spectrometer]
FFTpoints = {N}
FFTIntegrationTimeSec = {K * N / fs}
FFToverlapFactor = 2
WindowType = Cosine2
BandwidthHz = {fs / 2}
SourceFormat = Mark5B-1024-16-2
BitsPerSample = 2
SourceChannels = 16
UseFile1Channel = {ch}
ExtractPCal = 1
PCalOffsetHz = 0
BaseFilename1 = {tmp_path}/out
""")
    r = subprocess.run([str(PKG / "swspectrometer_gpu"), str(ini), str(data)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = np.fromfile(tmp_path / "out_swspec.bin", np.float32).reshape(nspec, N // 2 + 1)
    bins = np.fromfile(tmp_path / "out_pcal.bin", np.complex64).reshape(nspec, 32)
    planes = orc.unpack2bit(words.view(np.uint8), N * K * nspec, 16, orc.MARK5B_LUT)
    # one spectrum per call, like a reference core buffer that holds one spectrum
    for s in range(nspec):
        x = planes[ch - 1][s * N * K:(s + 1) * N * K]
        ref, ref_b = orc.spectrometer(x, N, 2, 2, K, 32, 32, 0.0, fs)
        assert np.linalg.norm(got[s] - ref[0]) / np.linalg.norm(ref[0]) < 1e-5
        assert np.linalg.norm(bins[s] - ref_b[0]) / np.linalg.norm(ref_b[0]) < 1e-5


def test_minicorrelator_cli_matches_oracle(cg, orc):
    r = subprocess.run([str(PKG / "minicorrelator_gpu"), "3", "8"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "Gbit/s" in r.stdout
    lines = [l for l in r.stdout.splitlines() if l.startswith(("auto", "baseline"))]
    assert len(lines) == 6
    # recompute the last integration of products (1,0) with the oracle
    S, N, raw_bytes, nint = 3, 1024, 256 * 16384, 8
    K = raw_bytes * 4 // N // nint
    raw = np.array([[(17 * i + 3 * j) % 256 for j in range(raw_bytes)] for i in range(S)], dtype=np.uint8)
    ref = orc.fx_fp32(raw, S, N, K, start_sample=(nint - 1) * K * N)
    line = [l for l in lines if "1-0" in l][0]
    nums = [float(x) for x in re.findall(r"[-+]?\d[\d.e+-]*", line.split(":")[1])]
    v = ref[orc.tri_index(1, 0)]
    assert np.allclose(nums[:4], v.real[:4], rtol=1e-4, atol=1e-3)
    assert np.allclose(nums[4:8], v.imag[:4], rtol=1e-4, atol=1e-3)


def test_swspectrometer_cli_two_sources(cg, orc, tmp_path):
    """Two input files: both auto spectra and the cross-polarisation spectrum."""
    import synth

    N, K, fs, nspec, nsub = 2048, 4, 32e6, 2, 4
    rng = np.random.default_rng(3)
    common = rng.standard_normal((N * K * nspec, nsub))
    files = []
    for f in range(2):
        x = 0.6 * common + 0.8 * rng.standard_normal(common.shape)
        raw = synth.pack2bit(synth.quantize_mark5b(x.astype(np.float32)).reshape(-1))
        path = tmp_path / f"src{f}.m5b"
        raw.tofile(path)
        files.append((path, raw))
    ini = tmp_path / "spec.ini"
    ini.write_text(f"""[Spectrometer]
FFTpoints = {N}
FFTIntegrationTimeSec = {K * N / fs}
FFToverlapFactor = 2
WindowType = Cosine2
BandwidthHz = {fs / 2}
SourceFormat = Mark5B-512-4-2
BitsPerSample = 2
SourceChannels = {nsub}
UseFile1Channel = 2
UseFile2Channel = 2
BaseFilename1 = {tmp_path}/out
""")
    r = subprocess.run([str(PKG / "swspectrometer_gpu"), str(ini), str(files[0][0]), str(files[1][0])],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    nb = N // 2 + 1
    a0 = np.fromfile(tmp_path / "out_swspec.bin", np.float32).reshape(nspec, nb)
    a1 = np.fromfile(tmp_path / "out_file2_swspec.bin", np.float32).reshape(nspec, nb)
    xp = np.fromfile(tmp_path / "out_xpol_swspec.bin", np.complex64).reshape(nspec, nb)
    for s in range(nspec):
        sl = slice(s * N * K, (s + 1) * N * K)
        x0 = orc.unpack2bit(files[0][1], N * K * nspec, nsub, orc.MARK5B_LUT)[1][sl]
        x1 = orc.unpack2bit(files[1][1], N * K * nspec, nsub, orc.MARK5B_LUT)[1][sl]
        rp, rx, _ = orc.spectrometer_xpol(x0, x1, N, 2, 2, K)
        assert np.linalg.norm(a0[s] - rp[0, 0]) / np.linalg.norm(rp[0, 0]) < 1e-5
        assert np.linalg.norm(a1[s] - rp[1, 0]) / np.linalg.norm(rp[1, 0]) < 1e-5
        assert np.linalg.norm(xp[s] - rx[0]) / np.linalg.norm(rx[0]) < 1e-5


def _spec_ini(tmp_path, N, K, fs, fmt, nsub, ch):
    ini = tmp_path / "spec.ini"
    ini.write_text(f"""[Spectrometer]
FFTpoints = {N}
FFTIntegrationTimeSec = {K * N / fs}
FFToverlapFactor = 2
WindowType = Cosine2
BandwidthHz = {fs / 2}
SourceFormat = {fmt}
BitsPerSample = 2
SourceChannels = {nsub}
UseFile1Channel = {ch}
ExtractPCal = 1
PCalOffsetHz = 0
BaseFilename1 = {tmp_path}/out
""")
    return ini


@pytest.mark.parametrize("fmt", ["Mark5B", "VDIF"])
def test_swspectrometer_cli_framed_recording(cg, orc, tmp_path, fmt):
    """SourceFormat = Mark5B / VDIF: a framed recording (headers, a blanked frame),
    headers stripped and blanking applied on the GPU; all spectra in one call."""
    import synth

    N, K, fs, nspec, nsub, ch = 4096, 8, 32e6, 3, 16, 5
    words, _ = synth.mark5b_subbands(16, N * K * nspec + 20000, fs_hz=fs, seed=41, n_channels=N // 2, pcal_amp=0.2)
    payload = words.view(np.uint8)
    if fmt == "Mark5B":
        nf = payload.size // 10000
        fr = synth.mark5b_frames(payload[: nf * 10000], prefix=777)
        synth.mark5b_fill(fr, 2, 0, 4000, prefix=777)
        good, planes = orc.mark5b_decode_framed(fr, nsub, N * K * nspec)
    else:
        mbps = int(fs * 2 * nsub / 1e6)
        nf = payload.size // 8000
        fr = synth.vdif_frames(payload[: nf * 8000], 8000, nsub, mbps, first_frame=5)
        synth.vdif_set_invalid(fr, 3, 8032)
        good, planes = orc.vdif_decode_framed(fr, nsub, mbps, N * K * nspec)
    assert good > 0
    data = tmp_path / "scan.bin"
    fr.tofile(data)
    ini = _spec_ini(tmp_path, N, K, fs, fmt, nsub, ch)
    r = subprocess.run([str(PKG / "swspectrometer_gpu"), str(ini), str(data)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = np.fromfile(tmp_path / "out_swspec.bin", np.float32).reshape(nspec, N // 2 + 1)
    bins = np.fromfile(tmp_path / "out_pcal.bin", np.complex64).reshape(nspec, 32)
    ref, ref_b = orc.spectrometer(planes[ch - 1], N, 2, 2, K, 32, 32, 0.0, fs)   # one call, all spectra
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-5
    assert np.linalg.norm(bins - ref_b) / np.linalg.norm(ref_b) < 1e-5
