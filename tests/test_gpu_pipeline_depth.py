"""Pipeline depth (K-stages of the shared-memory rings) changes timing only.

The autotuner picks the ring depth of each GEMM (tuning table: seventh column
for the FP64-accurate GEMMs, "f32" and "plain" entries, the "grouped" entry's
stage count); the environment overrides it (PHPC_STAGES for the tcgen05
engine, PHPC_DMMA_STAGES for the plain FP64 GEMM). Every depth must give the
bits of the default ring: the products and their summation order do not
depend on how many stages are in flight.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture
def inputs(torch_cuda, phpc):
    torch = torch_cuda
    m, k, n = 520, 1500, 700
    A = torch.empty((m, k), dtype=torch.float64, device="cuda")
    B = torch.empty((k, n), dtype=torch.float64, device="cuda")
    phpc.fill_wide_dev(A, m * k, 91, 0, -20, 20)
    phpc.fill_wide_dev(B, k * n, 92, 0, -20, 20)
    return m, k, n, A, B


@pytest.mark.parametrize("bn", ["128", "256"])
def test_modular_gemm_every_stage_count_same_bits(phpc, torch_cuda, monkeypatch, inputs, bn):
    torch = torch_cuda
    m, k, n, A, B = inputs
    q = 13
    monkeypatch.setenv("PHPC_OZAKI_BN", bn)
    ws = phpc.ozaki2_workspace_bytes(m, k, n, q)
    W = torch.empty(ws, dtype=torch.uint8, device="cuda")
    outs = {}
    for stages in ("0", "2", "3", "4", "5", "9"):  # 0: deepest; 9: more than fits, capped to the deepest
        if stages == "0":
            monkeypatch.delenv("PHPC_STAGES", raising=False)
        else:
            monkeypatch.setenv("PHPC_STAGES", stages)
        C = torch.zeros((m, n), dtype=torch.float64, device="cuda")
        phpc.dgemm_ozaki2_dev(m, k, n, A, k, B, n, C, n, q, W, ws)
        torch.cuda.synchronize()
        assert phpc.device_status() == 0
        outs[stages] = C
    for s, C in outs.items():
        assert torch.equal(C, outs["0"]), f"stages {s}"


@pytest.mark.parametrize("stages", ["2", "3", "5", "6"])
def test_plain_gemm_ring_depth_same_bits(phpc, torch_cuda, monkeypatch, inputs, stages):
    torch = torch_cuda
    m, k, n, A, B = inputs
    ref = torch.zeros((m, n), dtype=torch.float64, device="cuda")
    phpc.dgemm_dmma_dev(m, k, n, A, k, B, n, ref, n, 2, 2, 256)
    for tile in ("64", "128"):
        for pipe in ("dfma", "dmma"):
            monkeypatch.setenv("PHPC_DMMA_TILE", tile)
            monkeypatch.setenv("PHPC_FP64_PIPE", pipe)
            monkeypatch.setenv("PHPC_DMMA_STAGES", stages)
            C = torch.zeros((m, n), dtype=torch.float64, device="cuda")
            phpc.dgemm_dmma_dev(m, k, n, A, k, B, n, C, n, 2, 2, 256)
            torch.cuda.synchronize()
            assert phpc.device_status() == 0
            assert torch.equal(C, ref), (tile, pipe, stages)


def test_bf16x3_stage_counts_and_tiles_same_bits(phpc, torch_cuda, monkeypatch):
    torch = torch_cuda
    m, k, n = 640, 1100, 900
    g = torch.Generator(device="cuda").manual_seed(4)
    A = torch.randn((m, k), dtype=torch.float32, device="cuda", generator=g)
    B = torch.randn((k, n), dtype=torch.float32, device="cuda", generator=g)
    ws = phpc.bf16x3_workspace_bytes(m, k, n)
    W = torch.empty(ws, dtype=torch.uint8, device="cuda")
    outs = {}
    for bn, stages in (("256", "0"), ("256", "2"), ("256", "3"), ("128", "0"), ("128", "4")):
        monkeypatch.setenv("PHPC_F32_BN", bn)
        if stages == "0":
            monkeypatch.delenv("PHPC_STAGES", raising=False)
        else:
            monkeypatch.setenv("PHPC_STAGES", stages)
        C = torch.zeros((m, n), dtype=torch.float32, device="cuda")
        phpc.sgemm_bf16x3_dev(m, k, n, A, k, B, n, C, n, W, ws)
        torch.cuda.synchronize()
        assert phpc.device_status() == 0
        outs[(bn, stages)] = C
    for key, C in outs.items():
        if key[0] == "256":
            assert torch.equal(C, outs[("256", "0")]), key
        else:
            assert torch.equal(C, outs[("128", "0")]), key
    ref = A.double() @ B.double()
    err = float((outs[("256", "0")].double() - ref).norm() / ref.norm())
    assert err <= 2e-6


def test_grouped_stage_counts_same_bits(phpc, torch_cuda, monkeypatch):
    torch = torch_cuda
    shapes = phpc.grouped_shapes(40, seed=12, lo=32, hi=512)
    mats = []
    for i, (m, k, n) in enumerate(shapes):
        A = torch.empty((m, k), dtype=torch.float64, device="cuda")
        B = torch.empty((k, n), dtype=torch.float64, device="cuda")
        phpc.fill_wide_dev(A, m * k, 300 + 2 * i, 0, -20, 20)
        phpc.fill_wide_dev(B, k * n, 301 + 2 * i, 0, -20, 20)
        mats.append((A, B))
    results = []
    for stages in ("0", "2", "3"):
        if stages == "0":
            monkeypatch.delenv("PHPC_STAGES", raising=False)
        else:
            monkeypatch.setenv("PHPC_STAGES", stages)
        Cs = [torch.zeros((m, n), dtype=torch.float64, device="cuda") for m, k, n in shapes]
        probs = [(m, k, n, A, k, B, n, C, n) for (m, k, n), (A, B), C in zip(shapes, mats, Cs)]
        ws = phpc.GroupedPlan.workspace_bytes(probs, 0, moduli=13)
        W = torch.empty(ws, dtype=torch.uint8, device="cuda")
        plan = phpc.GroupedPlan(probs, 0, W, ws, moduli=13)
        plan.run()
        torch.cuda.synchronize()
        assert phpc.device_status() == 0
        plan.close()
        results.append(Cs)
    for Cs in results[1:]:
        for i, (C, C0) in enumerate(zip(Cs, results[0])):
            assert torch.equal(C, C0), i
    assert np.isfinite(results[0][0].cpu().numpy()).all()
