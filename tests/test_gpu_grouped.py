"""Grouped FP64-accurate GEMM (one plan, five launches, CUDA-graph replay).

Each problem of a grouped call must equal, bit for bit, the single-problem
Ozaki GEMM of the same inputs (the integer slice sums are exact whatever the
tiling, and the per-element fold order is the same), and stay within the
Ozaki bar against the double-double oracle.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def make_batch(torch, shapes, seed):
    rng = np.random.default_rng(seed)
    out = []
    for m, k, n in shapes:
        a = rng.uniform(-1, 1, (m, k)) * np.exp2(rng.integers(-20, 21, (m, k)))
        b = rng.uniform(-1, 1, (k, n)) * np.exp2(rng.integers(-20, 21, (k, n)))
        c0 = rng.uniform(-1, 1, (m, n))
        out.append((a, b, c0, *(torch.from_numpy(x).cuda() for x in (a, b, c0))))
    return out


def single(phpc, torch, A, B, C, s):
    m, k = A.shape
    n = B.shape[1]
    ws = phpc.ozaki_workspace_bytes(m, k, n, s)
    W = torch.empty(ws, dtype=torch.uint8, device="cuda")
    phpc.dgemm_ozaki_dev(m, k, n, A, k, B, n, C, n, s, W, ws)


@pytest.mark.parametrize("bn", ["128", "256"])
def test_grouped_equals_single(phpc, oracle, torch_cuda, monkeypatch, bn):
    torch = torch_cuda
    monkeypatch.setenv("PHPC_GROUPED_BN", bn)
    shapes = [(64, 64, 64), (16, 32, 48), (130, 70, 300), (7, 13, 5), (256, 1024, 128), (96, 2048, 80),
              (300, 17, 1), (1, 500, 260)] + phpc.grouped_shapes(12, seed=9, lo=16, hi=512)
    s = 7
    batch = make_batch(torch, shapes, 3)
    probs = [(A.shape[0], A.shape[1], B.shape[1], A, A.shape[1], B, B.shape[1], C, B.shape[1])
             for (_, _, _, A, B, C) in batch]
    ws = phpc.GroupedPlan.workspace_bytes(probs, s)
    W = torch.empty(ws, dtype=torch.uint8, device="cuda")
    plan = phpc.GroupedPlan(probs, s, W, ws)
    plan.run()
    torch.cuda.synchronize()
    assert phpc.device_status() == 0
    for i, (a, b, c0, A, B, C) in enumerate(batch):
        C1 = torch.from_numpy(c0).cuda()
        single(phpc, torch, A, B, C1, s)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(C.cpu().numpy(), C1.cpu().numpy(), err_msg=f"problem {i} {shapes[i]}")
        if i < 6:
            err = oracle.rel_errors(C.cpu().numpy(), oracle.gemm_dd(a, b, c0))
            assert err["frob"] <= 1e-14, (i, err)
    plan.close()


def test_graph_replay_accumulates(phpc, torch_cuda):
    torch = torch_cuda
    shapes = phpc.grouped_shapes(24, seed=2, lo=32, hi=384)
    s = 6
    batch = make_batch(torch, shapes, 4)
    probs = [(A.shape[0], A.shape[1], B.shape[1], A, A.shape[1], B, B.shape[1], C, B.shape[1])
             for (_, _, _, A, B, C) in batch]
    ws = phpc.GroupedPlan.workspace_bytes(probs, s)
    W = torch.empty(ws, dtype=torch.uint8, device="cuda")
    plan = phpc.GroupedPlan(probs, s, W, ws)
    plan.graph_launch()
    plan.graph_launch()  # C += A B twice
    torch.cuda.synchronize()
    assert phpc.device_status() == 0
    for i, (a, b, c0, A, B, C) in enumerate(batch):
        C2 = torch.from_numpy(c0).cuda()
        single(phpc, torch, A, B, C2, s)
        single(phpc, torch, A, B, C2, s)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(C.cpu().numpy(), C2.cpu().numpy(), err_msg=f"problem {i}")
    plan.close()


def test_plan_validation(phpc, torch_cuda):
    torch = torch_cuda
    A = torch.zeros(64, 64, dtype=torch.float64, device="cuda")
    probs = [(64, 64, 64, A, 64, A, 64, A, 64)]
    W = torch.empty(64, dtype=torch.uint8, device="cuda")
    with pytest.raises(phpc.PhpcError) as e:
        phpc.GroupedPlan(probs, 7, W, 64)
    assert e.value.code == 6
    with pytest.raises(phpc.PhpcError) as e:
        phpc.GroupedPlan([(0, 64, 64, A, 64, A, 64, A, 64)], 7, W, 64)
    assert e.value.code == 1


def single_modular(phpc, torch, A, B, C, q):
    """The single-problem modular call; returns its grids (ea, eb, ba, bb)."""
    m, k = A.shape
    n = B.shape[1]
    ws = phpc.ozaki2_workspace_bytes(m, k, n, q)
    W = torch.empty(ws, dtype=torch.uint8, device="cuda")
    phpc.dgemm_ozaki2_dev(m, k, n, A, k, B, n, C, n, q, W, ws)
    torch.cuda.synchronize()
    return phpc.ozaki2_grids(m, k, n, q, W, ws)


@pytest.mark.parametrize("bn", ["128", "256"])
def test_grouped_modular_equals_single(phpc, oracle, torch_cuda, monkeypatch, bn):
    """Modular plan: every problem bit-identical to the single-problem modular
    call (each with the grid width of its own K), and to the exact-integer
    model on the small ones."""
    import ozaki2_model

    torch = torch_cuda
    monkeypatch.setenv("PHPC_GROUPED_BN", bn)
    shapes = [(64, 64, 64), (16, 32, 48), (130, 70, 300), (7, 13, 5), (256, 1024, 128), (96, 2048, 80),
              (300, 17, 1), (1, 500, 260), (40, 2048, 72)] + phpc.grouped_shapes(12, seed=9, lo=16, hi=512)
    q = 15
    batch = make_batch(torch, shapes, 5)
    probs = [(A.shape[0], A.shape[1], B.shape[1], A, A.shape[1], B, B.shape[1], C, B.shape[1])
             for (_, _, _, A, B, C) in batch]
    ws = phpc.GroupedPlan.workspace_bytes(probs, 0, moduli=q)
    W = torch.empty(ws, dtype=torch.uint8, device="cuda")
    plan = phpc.GroupedPlan(probs, 0, W, ws, moduli=q)
    plan.run()
    torch.cuda.synchronize()
    assert phpc.device_status() == 0
    for i, (a, b, c0, A, B, C) in enumerate(batch):
        got = C.cpu().numpy()
        C1 = torch.from_numpy(c0).cuda()
        grid = single_modular(phpc, torch, A, B, C1, q)
        np.testing.assert_array_equal(got, C1.cpu().numpy(), err_msg=f"problem {i} {shapes[i]}")
        if a.size * b.shape[1] <= 200000:
            np.testing.assert_array_equal(got, ozaki2_model.gemm(a, b, c0, q, grid), err_msg=f"model, problem {i}")
        if i < 6:
            err = oracle.rel_errors(got, oracle.gemm_dd(a, b, c0))
            assert err["frob"] <= 1e-14, (i, err)
    plan.close()


def test_grouped_modular_graph_replay_and_validation(phpc, torch_cuda):
    torch = torch_cuda
    shapes = phpc.grouped_shapes(24, seed=2, lo=32, hi=384)
    q = 14
    batch = make_batch(torch, shapes, 6)
    probs = [(A.shape[0], A.shape[1], B.shape[1], A, A.shape[1], B, B.shape[1], C, B.shape[1])
             for (_, _, _, A, B, C) in batch]
    ws = phpc.GroupedPlan.workspace_bytes(probs, 0, moduli=q)
    W = torch.empty(ws, dtype=torch.uint8, device="cuda")
    plan = phpc.GroupedPlan(probs, 0, W, ws, moduli=q)
    plan.graph_launch()
    plan.graph_launch()  # C += A B twice
    torch.cuda.synchronize()
    assert phpc.device_status() == 0
    for i, (a, b, c0, A, B, C) in enumerate(batch):
        C2 = torch.from_numpy(c0).cuda()
        single_modular(phpc, torch, A, B, C2, q)
        single_modular(phpc, torch, A, B, C2, q)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(C.cpu().numpy(), C2.cpu().numpy(), err_msg=f"problem {i}")
    plan.close()
    with pytest.raises(phpc.PhpcError) as e:
        phpc.GroupedPlan(probs, 0, W, 64, moduli=q)
    assert e.value.code == 6
    with pytest.raises(phpc.PhpcError) as e:
        phpc.GroupedPlan(probs, 0, W, ws, moduli=17)
    assert e.value.code == 1


def test_grouped_512_problems_one_graph(phpc, oracle, torch_cuda):
    """The batching workload's size: 512 independent problems (m, k, n
    log-uniform in [64, 256], multiples of 16, seeded shapes), the modular plan
    with the benchmark's 13 moduli, run as one CUDA graph. Every problem is
    bit-identical to the single-problem modular call of the same inputs, and
    16 seeded problems stay within the FP64-accurate bar (1e-14) against the
    double-double oracle."""
    torch = torch_cuda
    shapes = phpc.grouped_shapes(512, seed=5, lo=64, hi=256)
    q = 13
    mats = []
    for i, (m, k, n) in enumerate(shapes):
        A = torch.empty((m, k), dtype=torch.float64, device="cuda")
        B = torch.empty((k, n), dtype=torch.float64, device="cuda")
        C = torch.empty((m, n), dtype=torch.float64, device="cuda")
        phpc.fill_wide_dev(A, m * k, 7000 + 3 * i, 0, -20, 20)
        phpc.fill_wide_dev(B, k * n, 7001 + 3 * i, 0, -20, 20)
        phpc.fill_uniform_dev(C, m * n, 7002 + 3 * i, 0)
        mats.append((A, B, C, C.clone()))
    probs = [(m, k, n, A, k, B, n, C, n) for (m, k, n), (A, B, C, _) in zip(shapes, mats)]
    ws = phpc.GroupedPlan.workspace_bytes(probs, 0, moduli=q)
    W = torch.empty(ws, dtype=torch.uint8, device="cuda")
    plan = phpc.GroupedPlan(probs, 0, W, ws, moduli=q)
    plan.graph_launch()
    torch.cuda.synchronize()
    assert phpc.device_status() == 0
    ws1 = max(phpc.ozaki2_workspace_bytes(m, k, n, q) for m, k, n in shapes)
    W1 = torch.empty(ws1, dtype=torch.uint8, device="cuda")
    for (m, k, n), (A, B, _, C1) in zip(shapes, mats):
        phpc.dgemm_ozaki2_dev(m, k, n, A, k, B, n, C1, n, q, W1, ws1)
    torch.cuda.synchronize()
    assert phpc.device_status() == 0
    for i, (_, _, C, C1) in enumerate(mats):
        assert torch.equal(C, C1), f"problem {i} {shapes[i]}"
    pick = np.random.default_rng(5).choice(512, size=16, replace=False)
    for i in sorted(int(x) for x in pick):
        A, B, C, _ = mats[i]
        c0 = torch.empty_like(C)
        phpc.fill_uniform_dev(c0, C.numel(), 7002 + 3 * i, 0)
        ref = oracle.gemm_dd(A.cpu().numpy(), B.cpu().numpy(), c0.cpu().numpy())
        err = oracle.rel_errors(C.cpu().numpy(), ref)
        assert err["frob"] <= 1e-14 and err["max"] <= 1e-14, (i, shapes[i], err)
    plan.close()



@pytest.mark.parametrize("scheme", ["modular", "digits"])
def test_grouped_unit_schedules_same_bits(phpc, torch_cuda, monkeypatch, scheme):
    """The grouped GEMM hands its work units out in order through a counter
    (the default) or assigns CTA c the units c, c + grid, ...
    (PHPC_GROUPED_SCHED=static): the same bits either way, over replays of
    the captured graph (the counter is zeroed before every launch)."""
    torch = torch_cuda
    shapes = phpc.grouped_shapes(60, seed=23, lo=16, hi=900)
    rng = np.random.default_rng(9)
    mats = [(torch.from_numpy(rng.uniform(-1, 1, (m, k)) * np.exp2(rng.integers(-20, 21, (m, k)))).cuda(),
             torch.from_numpy(rng.uniform(-1, 1, (k, n))).cuda()) for m, k, n in shapes]
    moduli, s = (13, 0) if scheme == "modular" else (0, 7)
    results = []
    for sched in ("static", "dynamic"):
        if sched == "static":
            monkeypatch.setenv("PHPC_GROUPED_SCHED", "static")
        else:
            monkeypatch.delenv("PHPC_GROUPED_SCHED", raising=False)
        Cs = [torch.zeros((m, n), dtype=torch.float64, device="cuda") for m, k, n in shapes]
        probs = [(m, k, n, A, k, B, n, C, n) for (m, k, n), (A, B), C in zip(shapes, mats, Cs)]
        ws = phpc.GroupedPlan.workspace_bytes(probs, s, moduli=moduli)
        W = torch.empty(ws, dtype=torch.uint8, device="cuda")
        plan = phpc.GroupedPlan(probs, s, W, ws, moduli=moduli)
        for _ in range(3):  # graph replays accumulate into C
            plan.graph_launch()
        torch.cuda.synchronize()
        assert phpc.device_status() == 0
        plan.close()
        results.append(Cs)
    for i, (C, C0) in enumerate(zip(results[1], results[0])):
        assert torch.equal(C, C0), i
