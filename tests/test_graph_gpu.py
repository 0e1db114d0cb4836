"""cellspe_fx_correlate_async on a caller's stream, captured into a CUDA graph.

After one call has sized the thread's workspace (and the first-use tables and
schedule choices exist), the asynchronous entry point issues only stream work,
so it can be captured and replayed; the replay must reproduce the blocking
call bit for bit.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", [0, 1])
def test_fx_async_graph_replay_matches_blocking_call(cg, mode):
    import torch

    import synth

    S, N, K = 16, 2048, 64
    raw = torch.from_numpy(synth.stations_offset_binary(S, N * K, rho=0.1, seed=7)).cuda()
    P = S * (S + 1) // 2
    ref = torch.zeros((N // 2, P), dtype=torch.complex64, device="cuda")
    p = cg.fx_params(S, N, K, raw.shape[1], x_mode=mode, memory=cg.MEM_DEVICE)
    cg.fx_correlate(p, raw, ref)
    s = torch.cuda.Stream()
    vis = torch.zeros_like(ref)
    with torch.cuda.stream(s):
        cg.fx_correlate_async(p, raw, vis, s.cuda_stream)          # sizes the workspace
    torch.cuda.synchronize()
    assert torch.equal(vis, ref)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s, capture_error_mode="relaxed"):
        cg.fx_correlate_async(p, raw, vis, torch.cuda.current_stream().cuda_stream)
    vis.zero_()
    torch.cuda.synchronize()
    for _ in range(2):
        g.replay()
    torch.cuda.synchronize()
    assert torch.equal(vis, ref)
