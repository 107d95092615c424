"""The value network's own kernels (the tcgen05 GEMM with FP32
accumulation in TMEM, pooling, loss, Adam) against an fp32 CPU restatement
of the same network: features exactly, logits and every gradient within BF16
tolerance (relative error <= 5e-2 and cosine >= 0.999 on each tensor), and a
training run that lowers the loss. The GEMM itself against an fp32 product
of the same bf16 operands over the shapes the network uses and ragged ones
(relative error <= 1e-2: fp32 accumulation, bf16 output rounding)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


def random_batch(n=96, seed=0, dev="cuda"):
    rng = np.random.default_rng(seed)
    ntask = 3
    Ts = np.array([10, 16, 32], dtype=np.int32)
    regs = rng.integers(0, 1 << 16, size=(n, 8, 32), dtype=np.uint16)
    regs[:, 0, :] = 0
    flags = rng.integers(0, 16, size=(n, 32), dtype=np.uint8)
    task = rng.integers(0, ntask, size=n).astype(np.uint16)
    for i in range(n):  # unused test slots are zero in engine states
        regs[i, :, Ts[task[i]]:] = 0
        flags[i, Ts[task[i]]:] = 0
    live = (rng.integers(0, 256, size=n) & 0xFE).astype(np.uint8)
    depth = rng.integers(0, 9, size=n).astype(np.uint8)
    task_io = rng.integers(0, 1 << 16, size=(ntask, 3, 32), dtype=np.uint16)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)  # noqa: E731
    # 16-bit tensors carry raw bits (the kernels read them as unsigned)
    return dict(regs=t(regs.astype(np.int16)), flags=t(flags), task=t(task.astype(np.int16)),
                live=t(live), depth=t(depth), task_io=t(task_io.astype(np.int16)),
                task_T=t(Ts), TP=32), (regs, flags, task, live, depth, task_io, Ts)


def cpu_features(regs, flags, task, task_io, Ts):
    n = regs.shape[0]
    X = np.zeros((n * 32, 176), dtype=np.float32)
    bits = np.arange(16)
    for i in range(n):
        T = Ts[task[i]]
        for t in range(T):
            row = X[i * 32 + t]
            for j in range(3):
                row[16 * j:16 * j + 16] = (int(task_io[task[i], j, t]) >> bits) & 1
            for r in range(1, 8):
                row[48 + 16 * (r - 1):48 + 16 * r] = (int(regs[i, r, t]) >> bits) & 1
            row[160:164] = (int(flags[i, t]) >> np.arange(4)) & 1
    return X


def rel(a, b):
    return float((a - b).norm() / max(b.norm(), 1e-12))


def cos(a, b):
    a, b = a.flatten().double(), b.flatten().double()
    return float(a @ b / max(a.norm() * b.norm(), 1e-30))


def test_features_exact():
    from pca_gb300.valuenet import ValueNet
    net = ValueNet()
    b, (regs, flags, task, live, depth, task_io, Ts) = random_batch(40)
    X = net.features(b["regs"], b["flags"], b["task"], 32, b["task_io"], b["task_T"])
    assert torch.equal(X.float().cpu(), torch.from_numpy(cpu_features(regs, flags, task, task_io, Ts)))


def test_forward_and_gradients_match_fp32():
    from pca_gb300.valuenet import ValueNet, reference_forward
    net = ValueNet(seed=3)
    b, (regs, flags, task, live, depth, task_io, Ts) = random_batch(96, seed=1)
    X = net.features(b["regs"], b["flags"], b["task"], 32, b["task_io"], b["task_T"])
    L = net.forward(X, b["live"], b["task"], b["task_T"], b["depth"])
    # reference on the CPU from the same bf16 weights and inputs
    W = {k: net.Wb[k].float().cpu().clone().requires_grad_() for k in net.W}
    bb = {k: v.cpu().clone().requires_grad_() for k, v in net.b.items()}
    Lr = reference_forward(W, bb, X.float().cpu(), torch.from_numpy(live),
                           torch.from_numpy(Ts), torch.from_numpy(task.astype(np.int64)),
                           torch.from_numpy(depth))
    assert rel(L.cpu(), Lr.detach()) < 5e-2
    g = torch.randn(96, 16, generator=torch.Generator().manual_seed(5))
    g = g.to(torch.bfloat16)
    grads = net.backward(g.cuda())
    (Lr * g.float()).sum().backward()
    for k in net.W:
        dW, db = grads[k]
        assert cos(dW.cpu(), W[k].grad) > 0.999, k
        assert rel(dW.cpu(), W[k].grad) < 5e-2, k
        assert cos(db.cpu(), bb[k].grad) > 0.999, k


def test_training_lowers_loss():
    from pca_gb300.valuenet import ValueNet
    net = ValueNet(seed=7, lr=1e-3, pos_weight=5.0)
    b, (regs, flags, task, live, depth, task_io, Ts) = random_batch(256, seed=2)
    # a learnable label: bit 3 of r1 on test 0
    label = ((regs[:, 1, 0] >> 3) & 1).astype(np.float32)
    b["label"] = torch.from_numpy(label).cuda()
    b["remaining"] = torch.from_numpy(np.where(label > 0, 2, -1).astype(np.int32)).cuda()
    first = net.train_step(b)
    for _ in range(150):
        last = net.train_step(b)
    assert last < 0.5 * first


def test_graph_step_matches_eager_steps():
    """The captured training step (one CUDA graph replay) updates the
    network exactly as the eager step does: every gradient is summed in a
    fixed order (split-K slabs, block partials), so after six steps the
    weights are the same bit for bit; the reported losses (fp32 sums over
    the batch) agree within rounding."""
    from pca_gb300.valuenet import ValueNet
    b, (regs, *_rest) = random_batch(200, seed=5)
    label = ((regs[:, 1, 0] >> 5) & 1).astype(np.float32)
    b["label"] = torch.from_numpy(label).cuda()
    b["remaining"] = torch.from_numpy(np.where(label > 0, 1, -1).astype(np.int32)).cuda()
    eager, graph = ValueNet(seed=11, lr=1e-3), ValueNet(seed=11, lr=1e-3)
    le = [float(eager.train_step(b)) for _ in range(6)]
    lg = [float(graph.train_step_graph(b)) for _ in range(6)]
    torch.cuda.synchronize()
    assert graph.step_n == eager.step_n == 6
    assert int(graph.step_dev.item()) == 6
    for name in eager.W:
        assert torch.equal(graph.W[name], eager.W[name]), name
        assert torch.equal(graph.b[name], eager.b[name]), name
    assert max(abs(a - c) for a, c in zip(le, lg)) < 1e-2 * max(abs(x) for x in le)


def _batch_tp(n, TP, seed):
    """States in a level layout of TP test columns (16 or 32)."""
    rng = np.random.default_rng(seed)
    Ts = np.array([3, 10, 16] if TP == 16 else [7, 16, 25, 32], dtype=np.int32)
    regs = rng.integers(0, 1 << 16, size=(n, 8, TP), dtype=np.uint16)
    regs[:, 0, :] = 0
    flags = rng.integers(0, 16, size=(n, TP), dtype=np.uint8)
    task = rng.integers(0, len(Ts), size=n).astype(np.uint16)
    for i in range(n):
        regs[i, :, Ts[task[i]]:] = 0
        flags[i, Ts[task[i]]:] = 0
    live = (rng.integers(0, 256, size=n) & 0xFE).astype(np.uint8)
    depth = rng.integers(0, 9, size=n).astype(np.uint8)
    task_io = rng.integers(0, 1 << 16, size=(len(Ts), 3, 32), dtype=np.uint16)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to("cuda")  # noqa: E731
    return (dict(regs=t(regs.astype(np.int16)), flags=t(flags), task=t(task.astype(np.int16)),
                 live=t(live), depth=t(depth), task_io=t(task_io.astype(np.int16)),
                 task_T=t(Ts)), (regs, flags, task, live, depth, task_io, Ts))


@pytest.mark.parametrize("TP,n", [(32, 203), (16, 61), (32, 5003)])
def test_fused_tcgen05_encoder_matches(TP, n):
    """The fused tcgen05 encoder (features -> E1 -> E2 -> pooling) against the
    unfused kernels and the fp32 CPU network: pooled rows within BF16
    rounding, logits within the same tolerance as the unfused path. n not a
    multiple of 4 leaves a partial last tile; n = 5003 gives each CTA several
    tiles (ring and barrier phases wrap)."""
    from pca_gb300.valuenet import ValueNet, reference_forward
    net = ValueNet(seed=5)
    b, (regs, flags, task, live, depth, task_io, Ts) = _batch_tp(n, TP, seed=TP + n)
    Pf = net.encode_pool(b["regs"], b["flags"], b["live"], b["task"], b["depth"], TP,
                         b["task_io"], b["task_T"])
    Lf = net.trunk(Pf)
    net.check_status()
    # unfused path on the same states (features need 32-column rows)
    regs32 = np.zeros((n, 8, 32), dtype=np.uint16)
    regs32[:, :, :TP] = regs
    flags32 = np.zeros((n, 32), dtype=np.uint8)
    flags32[:, :TP] = flags
    X = net.features(torch.from_numpy(regs32.astype(np.int16)).cuda(),
                     torch.from_numpy(flags32).cuda(), b["task"], 32, b["task_io"], b["task_T"])
    Lu = net.forward(X, b["live"], b["task"], b["task_T"], b["depth"])
    Pu = net._acts["P"]
    torch.cuda.synchronize()
    assert torch.isfinite(Pf.float()).all()
    assert rel(Pf.float().cpu(), Pu.float().cpu()) < 1e-2
    # columns 512.. (live bits, depth, zeros) are exact
    assert torch.equal(Pf[:, 512:].cpu(), Pu[:, 512:].cpu())
    assert rel(Lf.cpu(), Lu.cpu()) < 2e-2
    if n <= 256:
        W = {k: net.Wb[k].float().cpu() for k in net.W}
        bb = {k: v.cpu() for k, v in net.b.items()}
        Lr = reference_forward(W, bb, X.float().cpu(), torch.from_numpy(live),
                               torch.from_numpy(Ts), torch.from_numpy(task.astype(np.int64)),
                               torch.from_numpy(depth))
        assert rel(Lf.cpu(), Lr) < 5e-2
        assert cos(Lf[:, 0].cpu(), Lr[:, 0]) > 0.999


@pytest.mark.parametrize("M,N,K", [(128, 256, 64), (300, 176, 176), (262144 // 64, 256, 256),
                                   (8192, 528, 256), (8192, 16, 128), (777, 48, 16),
                                   (96, 256, 528)])
def test_tc_gemm_matches_fp32(M, N, K):
    """C = A . B^T (+ bias, ReLU) into bf16 and fp32, and the ReLU mask of an
    input gradient, against torch in fp32 on the same bf16 values."""
    import ctypes
    from pca_gb300.valuenet import _lib, _p
    lib = _lib()
    g = torch.Generator(device="cuda").manual_seed(M * 7 + N)
    A = torch.randn(M, K, device="cuda", generator=g).to(torch.bfloat16)
    B = torch.randn(N, K, device="cuda", generator=g).to(torch.bfloat16)
    bias = torch.randn(N, device="cuda", generator=g)
    mask = torch.randn(M, N, device="cuda", generator=g).to(torch.bfloat16)
    st = torch.zeros(1, device="cuda", dtype=torch.int32)
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    ref = A.float() @ B.float().t()
    Cb = torch.empty(M, N, device="cuda", dtype=torch.bfloat16)
    Cf = torch.empty(M, N, device="cuda", dtype=torch.float32)
    assert lib.pcagb_vnet_gemm_tc(_p(A), K, _p(B), K, _p(bias), None, 0, _p(Cb), _p(Cf), N, M, N,
                                  K, 1, 1, _p(st), s) == 0
    want = torch.relu(ref + bias)
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    assert rel(Cf, want) < 1e-4 and rel(Cb.float(), want) < 1e-2
    Cm = torch.empty(M, N, device="cuda", dtype=torch.bfloat16)
    assert lib.pcagb_vnet_gemm_tc(_p(A), K, _p(B), K, None, _p(mask), N, _p(Cm), None, N, M, N, K,
                                  0, 1, _p(st), s) == 0
    want = torch.where(mask.float() > 0, ref, torch.zeros_like(ref))
    torch.cuda.synchronize()
    assert rel(Cm.float(), want) < 1e-2


@pytest.mark.parametrize("splits", [1, 7, 64])
@pytest.mark.parametrize("out,inp", [(256, 176), (16, 128), (128, 256), (256, 528)])
def test_tc_weight_gradient_mn_major(splits, out, inp):
    """The weight gradient's form: dW = dY^T . X with dY [M][out] and X
    [M][in] read as stored (MN-major operands of the tcgen05 MMA, no
    transposes) and split-K fp32 adds, and db = the column sums of dY,
    against torch, on the network's layer shapes and a ragged batch."""
    import ctypes
    from pca_gb300.valuenet import _lib, _p
    lib = _lib()
    M = 4096 + 40
    g = torch.Generator(device="cuda").manual_seed(splits * 1000 + out + inp)
    dY = torch.randn(M, out, device="cuda", generator=g).to(torch.bfloat16)
    X = torch.randn(M, inp, device="cuda", generator=g).to(torch.bfloat16)
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    G = torch.zeros(out, inp, device="cuda", dtype=torch.float32)
    db = torch.zeros(out, device="cuda", dtype=torch.float32)
    st = torch.zeros(1, device="cuda", dtype=torch.int32)
    assert lib.pcagb_vnet_wgrad_tc(_p(dY), out, _p(X), inp, _p(G), inp, out, inp, M, splits,
                                   None, _p(st), s) == 0
    # the deterministic form: one slab per K split, summed in split order
    ns = lib.pcagb_vnet_wgrad_splits(M, splits)
    part = torch.empty(ns * out * inp, device="cuda", dtype=torch.float32)
    G2 = torch.zeros(out, inp, device="cuda", dtype=torch.float32)
    G3 = torch.zeros(out, inp, device="cuda", dtype=torch.float32)
    for Gd in (G2, G3):
        assert lib.pcagb_vnet_wgrad_tc(_p(dY), out, _p(X), inp, _p(Gd), inp, out, inp, M, splits,
                                       _p(part), _p(st), s) == 0
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    part = torch.empty(lib.pcagb_vnet_colsum_blocks(M, sms) * out, device="cuda",
                       dtype=torch.float32)
    assert lib.pcagb_vnet_colsum(_p(dY), M, out, out, _p(db), _p(part), sms, s) == 0
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    assert rel(G, dY.float().t() @ X.float()) < 1e-4
    assert rel(G2, dY.float().t() @ X.float()) < 1e-4
    assert torch.equal(G2, G3)
    assert rel(db, dY.float().sum(0)) < 1e-4


def test_adam_applies_each_layers_gradient():
    """Adam reads each layer's weight and bias gradients as the backward
    pass lays them out: the first step moves every weight by lr * g / (|g|
    + eps) against its gradient g."""
    from pca_gb300.valuenet import ValueNet
    net = ValueNet(seed=3, lr=1e-3)
    b, _ = random_batch(96, seed=1)
    X = net.features(b["regs"], b["flags"], b["task"], 32, b["task_io"], b["task_T"])
    net.forward(X, b["live"], b["task"], b["task_T"], b["depth"])
    gl = torch.randn(96, 16, generator=torch.Generator().manual_seed(5)).to(torch.bfloat16)
    grads = net.backward(gl.cuda())
    W0 = {k: net.W[k].clone() for k in net.W}
    b0 = {k: net.b[k].clone() for k in net.b}
    net.adam(grads)
    torch.cuda.synchronize()
    for k in net.W:
        dW, dbk = grads[k]
        want = W0[k] - 1e-3 * dW / (dW.abs() + 1e-8)
        cols = 521 if k == "T1" else want.shape[1]   # T1's padding columns stay zero
        assert rel(net.W[k][:, :cols], want[:, :cols]) < 1e-5, k
        assert rel(net.b[k], b0[k] - 1e-3 * dbk / (dbk.abs() + 1e-8)) < 1e-5, k
