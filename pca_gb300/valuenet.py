"""Value network: forward, backward and Adam on the GPU with the project's
own BF16 tensor-core kernels (pca_gb300/csrc/valuenet.cu).

torch provides device memory and the stream; every layer, gradient and
optimizer update is one of the C kernels, called through the C ABI.

Every matrix product runs on the fifth-generation tensor cores (TMA,
tcgen05.mma into TMEM, FP32 accumulation): the forward layers and the input
gradients (pcagb_vnet_gemm_tc, the ReLU derivative applied in the epilogue),
and the weight gradients (pcagb_vnet_wgrad_tc: split-K, both operands read
as stored, MN-major), whose bias gradients are the output gradients' column
sums (pcagb_vnet_colsum).

Network (the reference's ValueNetwork, python/model.py:16-84, with bit
features): per-test encoder 176 -> 256 -> 256 (ReLU), mean + max pooling
over the task's tests with the live mask and depth, trunk 528 -> 256 -> 128
(ReLU), head 128 -> 16 (column 0: can finish optimally; 1..9: remaining
steps). Loss: the reference's recipe (python/train.py:48-60): BCE with
pos_weight 50 on column 0 plus 0.5 x cross entropy on the positives.
"""
from __future__ import annotations

import ctypes
import math

import torch

from .pcalib import load_library

LAYERS = [("E1", 256, 176), ("E2", 256, 256), ("T1", 256, 528), ("T2", 128, 256),
          ("H", 16, 128)]
FEATURES = 176
ROWS = 32  # feature rows per state


def _lib():
    lib = load_library()
    vp, i, f = ctypes.c_void_p, ctypes.c_int, ctypes.c_float
    sz = ctypes.c_size_t
    sigs = {
        "pcagb_vnet_gemm_tc": [vp, i, vp, i, vp, vp, i, vp, vp, i, i, i, i, i, i, vp, vp],
        "pcagb_vnet_wgrad_tc": [vp, i, vp, i, vp, i, i, i, i, i, vp, vp, vp],
        "pcagb_vnet_wgrad_splits": [i, i],
        "pcagb_vnet_colsum": [vp, ctypes.c_longlong, i, i, vp, vp, i, vp],
        "pcagb_vnet_colsum_blocks": [ctypes.c_longlong, i],
        "pcagb_vnet_features": [vp, vp, vp, i, i, vp, vp, vp, vp],
        "pcagb_vnet_pool": [vp, vp, vp, vp, vp, i, vp, vp, vp],
        "pcagb_vnet_pool_bwd": [vp, vp, vp, vp, vp, i, vp, vp],
        "pcagb_vnet_loss": [vp, vp, vp, i, f, vp, vp, vp, vp],
        "pcagb_vnet_adam": [vp, vp, vp, vp, i, i, f, f, f, f, vp, vp, vp, vp],
        "pcagb_vnet_to_bf16": [vp, vp, sz, vp],
        "pcagb_vnet_encode_pool_tc": [vp, vp, vp, vp, vp, vp, vp, vp, vp, i, i, vp, vp, vp, vp,
                                      vp],
        "pcagb_vnet_gather_sample": [vp, vp, vp, vp, vp, vp, i, i, vp],
        "pcagb_vnet_compose_order": [vp, vp, i, vp, ctypes.c_ulonglong, vp],
    }
    for name, args in sigs.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = ctypes.c_int
    return lib


def _p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


class ValueNet:
    def __init__(self, device="cuda", seed=0, lr=3e-4, pos_weight=50.0):
        self.lib = _lib()
        self.dev = torch.device(device)
        self.lr, self.pos_weight = lr, pos_weight
        g = torch.Generator().manual_seed(seed)
        self.W, self.b, self.Wb, self.Wt = {}, {}, {}, {}
        self.mW, self.vW, self.mb, self.vb = {}, {}, {}, {}
        for name, out, inp in LAYERS:
            bound = 1.0 / math.sqrt(inp)
            w = (torch.rand(out, inp, generator=g) * 2 - 1) * bound
            if name == "T1":
                w[:, 521:] = 0.0  # padding columns of the trunk input
            self.W[name] = w.to(self.dev).contiguous()
            self.b[name] = ((torch.rand(out, generator=g) * 2 - 1) * bound).to(self.dev)
            for d in (self.mW, self.vW):
                d[name] = torch.zeros_like(self.W[name])
            for d in (self.mb, self.vb):
                d[name] = torch.zeros_like(self.b[name])
        self.step_n = 0
        self.step_dev = torch.zeros(1, device=self.dev, dtype=torch.int32)
        self._train_graphs = {}
        self._status = []
        self.sms = torch.cuda.get_device_properties(self.dev).multi_processor_count
        self._refresh_bf16()

    @property
    def stream(self):
        return ctypes.c_void_p(torch.cuda.current_stream(self.dev).cuda_stream)

    def _ck(self, rc):
        if rc != 0:
            raise RuntimeError(f"value-net kernel failed ({rc})")

    def _refresh_bf16(self):
        for name, out, inp in LAYERS:
            self.Wb[name] = self.W[name].to(torch.bfloat16).contiguous()
            self.Wt[name] = self.W[name].t().contiguous().to(torch.bfloat16)

    def n_params(self):
        return sum(w.numel() + self.b[k].numel() for k, w in self.W.items())

    # ---- kernels -----------------------------------------------------------
    def _status_word(self):
        """The status word every tcgen05 launch of this network reports a
        barrier time-out to (nonzero: the launch's result is void)."""
        if not self._status:
            self._status.append(torch.zeros(1, device=self.dev, dtype=torch.int32))
        return self._status[0]

    def _gemm(self, A, name, relu, out_f32=False, transposed=False, mask=None):
        """A[M,K] . W^T (+b), ReLU; or, for the input gradient, A[M,N] . W,
        zeroed where `mask` (the layer input's stored activation) is not
        positive. One tcgen05 GEMM (pcagb_vnet_gemm_tc)."""
        M, K = A.shape
        if transposed:
            B = self.Wt[name]          # [in][out]: rows are the output
            bias = None
        else:
            B = self.Wb[name]          # [out][in]
            bias = self.b[name]
        N = B.shape[0]
        C = torch.empty(M, N, device=self.dev, dtype=torch.float32 if out_f32 else torch.bfloat16)
        self._ck(self.lib.pcagb_vnet_gemm_tc(
            _p(A), A.stride(0), _p(B), B.stride(0), _p(bias), _p(mask),
            mask.stride(0) if mask is not None else 0, None if out_f32 else _p(C),
            _p(C) if out_f32 else None, N, M, N, K, int(relu), 1, _p(self._status_word()),
            self.stream))
        return C

    def _wgrad(self, dY, X, name):
        """dW = dY^T . X as one split-K tcgen05 GEMM reading dY [M][out] and
        X [M][in] as stored (MN-major operands, no transposes), and db =
        the column sums of dY."""
        out, inp = self.W[name].shape
        M = dY.shape[0]
        G = torch.zeros(out, inp, device=self.dev, dtype=torch.float32)
        db = torch.zeros(out, device=self.dev, dtype=torch.float32)
        bn = 256 if inp > 192 else (inp + 63) // 64 * 64
        tiles = ((out + 127) // 128) * ((inp + bn - 1) // bn)
        kblocks = (M + 63) // 64
        splits = self.lib.pcagb_vnet_wgrad_splits(
            M, max(1, min(kblocks, (2 * self.sms) // max(tiles, 1))))
        # each K split writes its own slab, added in split order: the same
        # gradients (and so the same network) on every run
        part = torch.empty(splits * out * inp, device=self.dev, dtype=torch.float32)
        self._ck(self.lib.pcagb_vnet_wgrad_tc(
            _p(dY), dY.stride(0), _p(X), X.stride(0), _p(G), inp, out, inp, M, splits, _p(part),
            _p(self._status_word()), self.stream))
        part = torch.empty(self.lib.pcagb_vnet_colsum_blocks(M, self.sms) * out,
                           device=self.dev, dtype=torch.float32)
        self._ck(self.lib.pcagb_vnet_colsum(_p(dY), M, out, dY.stride(0), _p(db), _p(part),
                                            self.sms, self.stream))
        return G, db

    def features(self, regs, flags, task, TP, task_io, task_T):
        n = task.shape[0]
        X = torch.empty(n * ROWS, FEATURES, device=self.dev, dtype=torch.bfloat16)
        self._ck(self.lib.pcagb_vnet_features(_p(regs), _p(flags), _p(task), TP, n, _p(task_io),
                                              _p(task_T), _p(X), self.stream))
        return X

    def forward(self, X, live, task, task_T, depth):
        n = task.shape[0]
        H1 = self._gemm(X, "E1", True)
        H2 = self._gemm(H1, "E2", True)
        P = torch.empty(n, 528, device=self.dev, dtype=torch.bfloat16)
        am = torch.empty(n, 256, device=self.dev, dtype=torch.uint8)
        self._ck(self.lib.pcagb_vnet_pool(_p(H2), _p(live), _p(task), _p(task_T), _p(depth), n,
                                          _p(P), _p(am), self.stream))
        Z1 = self._gemm(P, "T1", True)
        Z2 = self._gemm(Z1, "T2", True)
        L = self._gemm(Z2, "H", False, out_f32=True)
        self._acts = dict(X=X, H1=H1, H2=H2, P=P, am=am, Z1=Z1, Z2=Z2, task=task, task_T=task_T)
        return L

    def encode_pool(self, regs, flags, live, task, depth, TP, task_io, task_T):
        """Features -> E1 -> E2 -> pooling in one tcgen05 kernel (inference):
        the pooled rows P[n][528] without X, H1 or H2 in HBM."""
        n = task.shape[0]
        P = torch.empty(n, 528, device=self.dev, dtype=torch.bfloat16)
        status = self._status_word()
        self._ck(self.lib.pcagb_vnet_encode_pool_tc(
            _p(self.Wb["E1"]), _p(self.b["E1"]), _p(self.Wb["E2"]), _p(self.b["E2"]), _p(regs),
            _p(flags), _p(live), _p(task), _p(depth), TP, n, _p(task_io), _p(task_T), _p(P),
            _p(status), self.stream))
        return P

    def check_status(self):
        """Raise if a tcgen05 launch (fused encoder or GEMM) gave up on a
        barrier wait (reads the status words: synchronises with their
        stream)."""
        if not self._status:
            return
        v = int(self._status[0].item())
        self._status[0].zero_()
        if v:
            raise RuntimeError(f"tensor-core kernel aborted (barrier wait {v} timed out)")

    def trunk(self, P):
        Z1 = self._gemm(P, "T1", True)
        Z2 = self._gemm(Z1, "T2", True)
        return self._gemm(Z2, "H", False, out_f32=True)

    def forward_fused(self, regs, flags, live, task, depth, TP, task_io, task_T):
        """Logits [n][16] through the fused encoder and the trunk."""
        return self.trunk(self.encode_pool(regs, flags, live, task, depth, TP, task_io, task_T))

    def backward(self, dL):
        """dL: bf16 [n,16] gradient of the loss w.r.t. the logits. Returns
        {name: (dW, db)} in fp32."""
        a = self._acts
        grads = {}
        grads["H"] = self._wgrad(dL, a["Z2"], "H")
        dZ2 = self._gemm(dL, "H", False, transposed=True, mask=a["Z2"])
        grads["T2"] = self._wgrad(dZ2, a["Z1"], "T2")
        dZ1 = self._gemm(dZ2, "T2", False, transposed=True, mask=a["Z1"])
        grads["T1"] = self._wgrad(dZ1, a["P"], "T1")
        dP = self._gemm(dZ1, "T1", False, transposed=True)
        n = a["task"].shape[0]
        dH2 = torch.empty(n * ROWS, 256, device=self.dev, dtype=torch.bfloat16)
        self._ck(self.lib.pcagb_vnet_pool_bwd(_p(dP), _p(a["am"]), _p(a["task"]),
                                              _p(a["task_T"]), _p(a["H2"]), n, _p(dH2),
                                              self.stream))
        grads["E2"] = self._wgrad(dH2, a["H1"], "E2")
        dH1 = self._gemm(dH2, "E2", False, transposed=True, mask=a["H1"])
        grads["E1"] = self._wgrad(dH1, a["X"], "E1")
        return grads

    def loss(self, L, label, remaining):
        """The loss (a device scalar: nothing is read back) and its
        gradient w.r.t. the logits."""
        n = L.shape[0]
        dL = torch.empty(n, 16, device=self.dev, dtype=torch.bfloat16)
        stats = torch.zeros(3, device=self.dev, dtype=torch.float32)
        npos = (label > 0.5).sum(dtype=torch.float32).reshape(1)
        self._ck(self.lib.pcagb_vnet_loss(_p(L), _p(label), _p(remaining), n, self.pos_weight,
                                          _p(npos), _p(dL), _p(stats), self.stream))
        loss = stats[0] / n + 0.5 * stats[1] / npos[0].clamp(min=1.0)
        return loss, dL

    def adam(self, grads, b1=0.9, b2=0.999, eps=1e-8):
        self.step_n += 1
        self.step_dev += 1
        for name, out, inp in LAYERS:
            G, gb = grads[name]
            self._ck(self.lib.pcagb_vnet_adam(_p(self.W[name]), _p(G), _p(self.mW[name]),
                                              _p(self.vW[name]), out, inp, self.lr, b1, b2, eps,
                                              _p(self.step_dev), _p(self.Wb[name]),
                                              _p(self.Wt[name]), self.stream))
            self._ck(self.lib.pcagb_vnet_adam(_p(self.b[name]), _p(gb), _p(self.mb[name]),
                                              _p(self.vb[name]), 1, out, self.lr, b1, b2, eps,
                                              _p(self.step_dev), None, None, self.stream))
        with torch.no_grad():
            self.W["T1"][:, 521:] = 0.0
            self.Wb["T1"][:, 521:] = 0.0
            self.Wt["T1"][521:, :] = 0.0

    def train_step(self, batch):
        """One step on a batch dict (device tensors): regs, flags, live, task,
        task_io, task_T, TP, depth (uint8 per state), label, remaining.
        Returns the loss as a device scalar."""
        X = self.features(batch["regs"], batch["flags"], batch["task"], batch["TP"],
                          batch["task_io"], batch["task_T"])
        L = self.forward(X, batch["live"], batch["task"], batch["task_T"], batch["depth"])
        loss, dL = self.loss(L, batch["label"], batch["remaining"])
        self.adam(self.backward(dL))
        return loss

    BATCH_KEYS = ("regs", "flags", "live", "task", "task_io", "task_T", "depth", "label",
                  "remaining")

    def train_step_graph(self, batch):
        """train_step as one CUDA graph replay: the step (features, forward,
        loss, backward, Adam: about sixty launches) is captured once per
        batch shape into static buffers, and each call copies the batch in
        and replays it. Returns the loss as a device scalar."""
        key = (batch["task"].shape[0], batch["task_io"].shape[0], batch["TP"])
        G = self._train_graphs.get(key)
        if G is None:
            static = {k: batch[k].clone() for k in self.BATCH_KEYS}
            static["TP"] = batch["TP"]
            side = torch.cuda.Stream(device=self.dev)
            side.wait_stream(torch.cuda.current_stream(self.dev))
            with torch.cuda.stream(side):
                first = self.train_step(static)   # this call's step, outside the capture
            torch.cuda.current_stream(self.dev).wait_stream(side)
            graph = torch.cuda.CUDAGraph()
            with torch.cuda.graph(graph, stream=side):
                loss = self.train_step(static)
            torch.cuda.current_stream(self.dev).wait_stream(side)
            # the capture recorded a step without running it
            self.step_n -= 1
            self._train_graphs[key] = {"graph": graph, "static": static, "loss": loss}
            return first
        for k in self.BATCH_KEYS:
            G["static"][k].copy_(batch[k])
        G["graph"].replay()
        self.step_n += 1
        return G["loss"].clone()

    def score(self, regs, flags, live, task, task_io, task_T, TP, depth):
        X = self.features(regs, flags, task, TP, task_io, task_T)
        return self.forward(X, live, task, task_T, depth)[:, 0]

    def state_dict(self):
        return {k: v.detach().cpu() for k, v in {**{"W." + n: w for n, w in self.W.items()},
                                                  **{"b." + n: b for n, b in self.b.items()}}.items()}

    def load_state_dict(self, sd):
        for k, v in sd.items():
            kind, name = k.split(".", 1)
            (self.W if kind == "W" else self.b)[name].copy_(v.to(self.dev))
        self._refresh_bf16()


def reference_forward(W, b, X, live, task_T, task, depth, bf16=True):
    """fp32 CPU restatement of the same network (for gradient checks): X
    [n*32,176], returns logits [n,16]; autograd-ready when W/b require grad.
    With bf16=True the activations (and, through autograd, their gradients)
    are rounded to bf16 where the kernels store them."""
    r = (lambda x: x.to(torch.bfloat16).float()) if bf16 else (lambda x: x)
    n = live.shape[0]
    H1 = r(torch.relu(X @ W["E1"].t() + b["E1"]))
    H2 = r(torch.relu(H1 @ W["E2"].t() + b["E2"])).view(n, ROWS, 256)
    T = task_T[task].long()
    mask = (torch.arange(ROWS)[None, :] < T[:, None]).float()
    mean = (H2 * mask[:, :, None]).sum(1) / T[:, None].float()
    mx = torch.where(mask[:, :, None] > 0, H2, torch.full_like(H2, -1e30)).max(1).values
    g = torch.zeros(n, 16)
    g[:, :8] = ((live.long()[:, None] >> torch.arange(8)[None, :]) & 1).float()
    g[:, 8] = depth.float()
    P = r(torch.cat([mean, mx, g], 1))
    Z1 = r(torch.relu(P @ W["T1"].t() + b["T1"]))
    Z2 = r(torch.relu(Z1 @ W["T2"].t() + b["T2"]))
    return Z2 @ W["H"].t() + b["H"]
