"""The engine's reference layout (RG_RNG_XORWOW_REF) against the reference's
own GPU kernel, monte_carlo_kernel of src/05-GPU/monte_carlos_cuda.cu:23-72,
compiled unmodified for sm_103a from the reference's source (oracle/Makefile,
target refcuda) and launched as its host wrapper launches it (.cu:121-128).

Both kernels get the same FP64 factor (the engine's own Cholesky) and the same
seed; both call curand_init(seed, path, 0) and curand_normal_double.  The
reference accumulates R in FP64, the engine in FP32, so S per path must be
identical except on paths where some asset return lies within NEAR = 2e-6 of
the threshold (|R_i + x| < NEAR in FP64, checked path by path with the
oracle's FP64 arithmetic on cuRAND's normals).  The workload is the drop-in
one: N = 50 one-factor assets, x = 3%, k = 5, seed 67, at the full M = 1e8.

The fatbin is built where the reference tree is present; elsewhere these
tests are skipped.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NEAR = 2e-6


@pytest.fixture(scope="module")
def refk(oracle):
    if not oracle.ref_kernel_available():
        pytest.skip("the reference's kernel is compiled only where the reference tree is present "
                    "(make -C oracle refcuda)")
    return oracle


def _both(gpu, refk, M, path_check=200):
    import torch
    from riskgpu import synth
    p = synth.one_factor_50(n_paths=M)
    port = gpu.Portfolio(p.mu, p.sigma)
    L = np.ascontiguousarray(port.factor())
    dev = torch.device("cuda")
    d_mu = torch.tensor(p.mu, dtype=torch.float64, device=dev)
    d_L = torch.tensor(L, dtype=torch.float64, device=dev)
    S_ref = torch.full((M,), -1, dtype=torch.int32, device=dev)
    cnt = torch.zeros(1, dtype=torch.int32, device=dev)
    torch.cuda.synchronize()
    ms = refk.ref_kernel_run(M, p.n, p.k, p.x, d_mu.data_ptr(), d_L.data_ptr(), p.seed, S_ref.data_ptr(),
                             cnt.data_ptr())
    S_eng = torch.full((M,), -2, dtype=torch.int32, device=dev)
    q = gpu.make_query(M, p.seed, x=p.x, k=p.k, horizon=1, port_threshold=-1.0, rng=gpu.RNG_XORWOW_REF,
                       d_s_values=S_eng.data_ptr())
    res = port.simulate(q)
    torch.cuda.synchronize()
    diff = torch.nonzero(S_eng != S_ref).flatten().cpu().numpy()
    ref_count = int(cnt.item())
    # counts of S >= k over the paths where the two kernels agree are equal by
    # construction; check the engine's count against its own S, and the
    # reference's atomic count against its S
    assert res["crash_count"] == int((S_eng >= p.k).sum().item())
    assert ref_count == int((S_ref >= p.k).sum().item())
    # every differing path lies within NEAR of the threshold (FP64 oracle on
    # cuRAND's normals for that path)
    for idx in diff[:path_check]:
        Z = refk.curand_xorwow_normals(p.seed, 1, p.n, path0=int(idx))
        _, S1, R1 = refk.kernel_from_normals(p.mu, L, Z, p.x, p.k, return_R=True)
        assert int(S1[0]) == int(S_ref[int(idx)].item()), "the oracle disagrees with the reference kernel"
        assert np.min(np.abs(R1[0] + p.x)) < NEAR, f"path {idx} differs away from the threshold"
    port.close()
    return dict(M=M, ms=ms, diff=len(diff), ref_count=ref_count, eng_count=res["crash_count"],
                S_ref=S_ref, S_eng=S_eng)


def test_reference_kernel_slices_match_oracle(gpu, refk):
    """Per-path S of the reference kernel itself equals the oracle's FP64
    restatement on cuRAND's normals (away from the threshold), on a slice."""
    r = _both(gpu, refk, 20_000)
    Z = refk.curand_xorwow_normals(67, 20_000, 50)
    from riskgpu import synth
    p = synth.one_factor_50(n_paths=1)
    port = gpu.Portfolio(p.mu, p.sigma)
    L = port.factor()
    _, S_or, R_or = refk.kernel_from_normals(p.mu, L, Z, p.x, p.k, return_R=True)
    near = np.min(np.abs(R_or + p.x), axis=1) < NEAR
    S_ref = r["S_ref"].cpu().numpy()
    assert not ((S_ref != S_or) & ~near).any()
    assert r["diff"] <= int(near.sum())


def test_full_count_at_1e8_matches_reference_kernel(gpu, refk):
    """The drop-in workload at its full size: S on all 1e8 paths and the
    count of S >= k agree with the reference kernel, except on paths within
    NEAR of the threshold (each differing path is checked, up to 200)."""
    r = _both(gpu, refk, 100_000_000, path_check=200)
    # paths near the threshold are rare: at most 1e-5 of all paths differ
    assert r["diff"] <= 1000, r["diff"]
    assert abs(r["ref_count"] - r["eng_count"]) <= r["diff"]
    # the last slice of the range, path by path (indices near 1e8)
    tail = slice(100_000_000 - 4096, 100_000_000)
    assert (r["S_ref"][tail] != r["S_eng"][tail]).sum().item() <= r["diff"]
