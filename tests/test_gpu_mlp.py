"""GPU: the learned proposer's hand-written kernels against the FP64 CPU
restatement (oracle/mlp.py): forward pass, BF16 inference, gradients (the
gradient check), and that training lowers the loss."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _mlp(gb, seed=3):
    m = gb.GbMlp()
    assert gb.lib().gb_mlp_init(C.byref(m), seed) == 0
    rng = np.random.default_rng(seed)
    for k in range(16):
        m.in_mean[k] = float(rng.normal())
        m.in_scale[k] = float(rng.uniform(0.5, 2.0))
    for k in range(64):
        m.b1[k] = float(rng.normal() * 0.1)
        m.b2[k] = float(rng.normal() * 0.1)
    m.b3 = 0.05
    m.out_scale = 0.7
    m.out_bias = -0.2
    return m


def _dev(torch, m):
    buf = torch.empty(C.sizeof(m), dtype=torch.uint8, device="cuda")
    buf.copy_(torch.frombuffer(bytearray(bytes(m)), dtype=torch.uint8))
    return buf


def test_forward_and_bf16_inference(gb, torch_cuda):
    from oracle import mlp as om
    torch = torch_cuda
    m = _mlp(gb)
    p = om.unpack(m)
    x = np.random.default_rng(1).normal(size=(777, 16)).astype(np.float32)
    ref, _ = om.forward(p, x.astype(np.float64))
    w = _dev(torch, m)
    xd = torch.as_tensor(x, device="cuda")
    y = torch.empty(777, dtype=torch.float32, device="cuda")
    assert gb.lib().gb_mlp_forward_f32(w.data_ptr(), xd.data_ptr(), y.data_ptr(), 777, None,
                                       None) == 0
    np.testing.assert_allclose(y.cpu().numpy(), ref, rtol=1e-4, atol=1e-5)
    # BF16 weights, FP32 accumulation: against the FP64 model with BF16-rounded weights
    pb = dict(p)
    for k in ("w1", "w2", "w3"):
        pb[k] = om.bf16_round(p[k])
    refb, _ = om.forward(pb, x.astype(np.float64))
    assert gb.lib().gb_mlp_infer_bf16(w.data_ptr(), xd.data_ptr(), y.data_ptr(), 777, None) == 0
    np.testing.assert_allclose(y.cpu().numpy(), refb, rtol=1e-4, atol=1e-5)


def test_gradients_match_fp64_oracle(gb, torch_cuda):
    from oracle import mlp as om
    torch = torch_cuda
    m = _mlp(gb, 7)
    p = om.unpack(m)
    B = 513
    rng = np.random.default_rng(2)
    x = rng.normal(size=(B, 16)).astype(np.float32)
    dy = rng.normal(size=B).astype(np.float32)
    g_ref = om.backward(p, x.astype(np.float64), dy.astype(np.float64))
    w = _dev(torch, m)
    xd = torch.as_tensor(x, device="cuda")
    dyd = torch.as_tensor(dy, device="cuda")
    y = torch.empty(B, dtype=torch.float32, device="cuda")
    act = torch.empty(gb.lib().gb_mlp_act_floats(B), dtype=torch.float32, device="cuda")
    work = torch.empty(gb.lib().gb_mlp_backward_workspace_bytes(B), dtype=torch.uint8,
                       device="cuda")
    G = torch.empty(C.sizeof(gb.GbMlp), dtype=torch.uint8, device="cuda")
    L = gb.lib()
    assert L.gb_mlp_forward_f32(w.data_ptr(), xd.data_ptr(), y.data_ptr(), B, act.data_ptr(),
                                None) == 0
    assert L.gb_mlp_backward_f32(w.data_ptr(), xd.data_ptr(), act.data_ptr(), dyd.data_ptr(),
                                 G.data_ptr(), B, work.data_ptr(), None) == 0
    torch.cuda.synchronize()
    g = om.unpack(gb.GbMlp.from_buffer_copy(bytes(G.cpu().numpy().tobytes())))
    for k in ("w1", "b1", "w2", "b2", "w3"):
        err = np.max(np.abs(g[k] - g_ref[k])) / max(np.max(np.abs(g_ref[k])), 1e-12)
        assert err < 1e-4, (k, err)
    assert g["b3"] == pytest.approx(g_ref["b3"], rel=1e-4)
    # and against a central finite difference of the FP64 model on one weight
    eps = 1e-6
    p2 = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in p.items()}
    p2["w2"][3, 5] += eps
    fp, _ = om.forward(p2, x.astype(np.float64))
    p2["w2"][3, 5] -= 2 * eps
    fm, _ = om.forward(p2, x.astype(np.float64))
    fd = float(np.dot(dy, (fp - fm) / (2 * eps)))
    assert g["w2"][3, 5] == pytest.approx(fd, rel=1e-3, abs=1e-6)


def test_training_lowers_loss(gb, torch_cuda):
    from ode_prototyping_gb300 import learned
    rng = np.random.default_rng(4)
    x = rng.normal(size=(2048, 16)).astype(np.float32)
    y = (0.3 * np.tanh(x[:, 0] - 0.5 * x[:, 3]) + 0.1 * x[:, 5]).astype(np.float32)
    m0, loss0 = learned.train(x, y, epochs=1, lr=1e-3)
    m1, loss1 = learned.train(x, y, epochs=600, lr=3e-3)
    assert loss1 < 0.2 * loss0, (loss0, loss1)
