"""The warm-start network's kernels against the CPU oracle, torch-CPU conv3d and autograd.

Inputs and weights are rounded to bf16 first; the oracle then computes in float64, so what is
left is the kernels' FP32 accumulation and the bf16 rounding of their outputs:
  - activations (bf16 out): 1e-2 norm-wise relative (bf16 has an 8-bit mantissa);
  - weight / bias gradients (FP32 out): 1e-4;
  - the whole network: each layer's backward in place as tight as above; end to end, 0.15 per
    layer against an independent float64 autograd of the network that rounds activations and
    their gradients to bf16 where the kernels store them (rounding decisions that go the other
    way multiply through the layers)."""

import ctypes as C

import numpy as np
import pytest

import conftest
from conftest import rel_err

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
F = torch.nn.functional

TOL_ACT = 1e-2
TOL_WGRAD = 1e-4
TOL_NET = 0.15


def _ws():
    return conftest.load_package().warmstart


def bf(a):
    """numpy float -> bf16-representable float64 torch CPU tensor"""
    return torch.from_numpy(np.asarray(a, np.float32)).to(torch.bfloat16).to(torch.float64)


def dev(t):
    return t.to(torch.bfloat16).cuda().contiguous()


def up2(a):  # (z, y, x, c) nearest upsampling
    return a.repeat_interleave(2, 0).repeat_interleave(2, 1).repeat_interleave(2, 2)


def conv_ref(x, w, b=None):
    """x (z, y, x, ci) float64; w [co][27][ci] -> (z, y, x, co), zero padding"""
    co, _, ci = w.shape
    wt = w.reshape(co, 3, 3, 3, ci).permute(0, 4, 1, 2, 3)
    y = F.conv3d(x.permute(3, 0, 1, 2)[None], wt, b, padding=1)
    return y[0].permute(1, 2, 3, 0)


def _pack(L, w, cin, cout):
    nb = L.el_nn_packed_weight_bytes(cin, cout) // 2
    fwd = torch.empty(nb, dtype=torch.bfloat16, device="cuda")
    bwd = torch.empty(nb, dtype=torch.bfloat16, device="cuda")
    wd = torch.from_numpy(np.asarray(w, np.float32)).cuda()
    assert L.el_nn_pack_weights(cin, cout, wd.data_ptr(), fwd.data_ptr(), bwd.data_ptr(), None) == 0
    return fwd, bwd


def _args(W, shape, cin, cout, a, ca, up, b=None, cb=0):
    args = W.ConvArgs()
    args.nx, args.ny, args.nz = shape
    args.cin, args.cout = cin, cout
    args.in_a, args.ca, args.upsample_a = a.data_ptr(), ca, up
    args.in_b, args.cb = (b.data_ptr() if b is not None else None), cb
    return args


def _rand(rng, *shape, scale=1.0):
    return rng.standard_normal(shape).astype(np.float32) * scale


@pytest.mark.parametrize("cin,cout,shape", [(16, 16, (20, 9, 5)), (32, 64, (16, 16, 4)), (64, 128, (16, 8, 3))])
def test_conv_forward_matches_conv3d(cin, cout, shape):
    W = _ws()
    L = W.lib()
    rng = np.random.default_rng(cin + cout)
    nx, ny, nz = shape
    x = bf(_rand(rng, nz, ny, nx, cin))
    w = bf(_rand(rng, cout, 27, cin, scale=(2.0 / (27 * cin)) ** 0.5))
    bias = torch.from_numpy(_rand(rng, cout, scale=0.1)).to(torch.float64)
    fwd, _ = _pack(L, w.numpy(), cin, cout)
    xd = dev(x)
    out = torch.empty((nz, ny, nx, cout), dtype=torch.bfloat16, device="cuda")
    bd = bias.float().cuda()
    args = _args(W, shape, cin, cout, xd, cin, 0)
    args.weights, args.bias, args.relu = fwd.data_ptr(), bd.data_ptr(), 1
    args.out_a, args.out_a_channels = out.data_ptr(), cout
    assert L.el_nn_conv3_forward(C.byref(args), None) == 0
    torch.cuda.synchronize()
    ref = torch.relu(conv_ref(x, w, bias.float().double()))
    assert rel_err(out.float().cpu().numpy(), ref.numpy()) < TOL_ACT


def test_conv_forward_concat_upsample_and_split_output():
    W = _ws()
    L = W.lib()
    rng = np.random.default_rng(3)
    nx, ny, nz = 16, 16, 8
    a = bf(_rand(rng, nz // 2, ny // 2, nx // 2, 64))
    b = bf(_rand(rng, nz, ny, nx, 32))
    w = bf(_rand(rng, 32, 27, 96, scale=0.05))
    fwd, _ = _pack(L, w.numpy(), 96, 32)
    out_a = torch.empty((nz, ny, nx, 16), dtype=torch.bfloat16, device="cuda")
    out_b = torch.empty((nz, ny, nx, 16), dtype=torch.bfloat16, device="cuda")
    ad, bd = dev(a), dev(b)
    args = _args(W, (nx, ny, nz), 96, 32, ad, 64, 1, bd, 32)
    args.weights, args.relu = fwd.data_ptr(), 0
    args.out_a, args.out_a_channels, args.out_b = out_a.data_ptr(), 16, out_b.data_ptr()
    assert L.el_nn_conv3_forward(C.byref(args), None) == 0
    torch.cuda.synchronize()
    ref = conv_ref(torch.cat([up2(a), b], dim=3), w)
    got = torch.cat([out_a.float().cpu(), out_b.float().cpu()], dim=3)
    assert rel_err(got.numpy(), ref.numpy()) < TOL_ACT


def test_conv_backward_data_and_weight_match_autograd():
    """A decoder layer: y = relu(conv([up(a), b])); gradients of sum(g * y)."""
    W = _ws()
    L = W.lib()
    rng = np.random.default_rng(5)
    nx, ny, nz = 16, 8, 6
    ca, cb, cout = 64, 32, 32
    cin = ca + cb
    a = bf(_rand(rng, nz // 2, ny // 2, nx // 2, ca))
    b = bf(_rand(rng, nz, ny, nx, cb))
    w = bf(_rand(rng, cout, 27, cin, scale=0.05))
    bias = torch.from_numpy(_rand(rng, cout, scale=0.05))
    g = bf(_rand(rng, nz, ny, nx, cout))
    fwd, bwd = _pack(L, w.numpy(), cin, cout)
    ad, bd, gd, biasd = dev(a), dev(b), dev(g), bias.cuda()
    y = torch.empty((nz, ny, nx, cout), dtype=torch.bfloat16, device="cuda")
    args = _args(W, (nx, ny, nz), cin, cout, ad, ca, 1, bd, cb)
    args.weights, args.bias, args.relu = fwd.data_ptr(), biasd.data_ptr(), 1
    args.out_a, args.out_a_channels = y.data_ptr(), cout
    assert L.el_nn_conv3_forward(C.byref(args), None) == 0
    # backward data: conv of g masked by y > 0 with the backward packing, split into the inputs
    gup = torch.empty((nz, ny, nx, ca), dtype=torch.bfloat16, device="cuda")
    gb = torch.empty((nz, ny, nx, cb), dtype=torch.bfloat16, device="cuda")
    ga = torch.empty((nz // 2, ny // 2, nx // 2, ca), dtype=torch.bfloat16, device="cuda")
    d = _args(W, (nx, ny, nz), cout, cin, gd, cout, 0)
    d.mask, d.weights, d.relu = y.data_ptr(), bwd.data_ptr(), 0
    d.out_a, d.out_a_channels, d.out_b = gup.data_ptr(), ca, gb.data_ptr()
    assert L.el_nn_conv3_forward(C.byref(d), None) == 0
    assert L.el_nn_gather8(nx, ny, nz, ca, gup.data_ptr(), ga.data_ptr(), None) == 0
    # backward weight
    dw = torch.zeros(cout * 27 * cin, dtype=torch.float32, device="cuda")
    db = torch.zeros(cout, dtype=torch.float32, device="cuda")
    wsz = L.el_nn_conv3_backward_weight_workspace(nx, ny, nz, cin, cout)
    ws = torch.empty(wsz // 4 + 1, dtype=torch.float32, device="cuda")
    args.out_a = y.data_ptr()
    assert L.el_nn_conv3_backward_weight(C.byref(args), gd.data_ptr(), dw.data_ptr(), db.data_ptr(), ws.data_ptr(),
                                         wsz, None) == 0
    torch.cuda.synchronize()
    # oracle: the same mask (our y > 0), float64 autograd of the linear part
    mask = (y.float().cpu() > 0).double()
    gm = g * mask
    a_ = a.clone().requires_grad_(True)
    b_ = b.clone().requires_grad_(True)
    w_ = w.clone().requires_grad_(True)
    z = conv_ref(torch.cat([up2(a_), b_], dim=3), w_)
    (z * gm).sum().backward()
    assert rel_err(ga.float().cpu().numpy(), a_.grad.numpy()) < TOL_ACT
    assert rel_err(gb.float().cpu().numpy(), b_.grad.numpy()) < TOL_ACT
    assert rel_err(dw.cpu().numpy().reshape(cout, 27, cin), w_.grad.numpy()) < TOL_WGRAD
    assert rel_err(db.cpu().numpy(), gm.sum(dim=(0, 1, 2)).numpy()) < TOL_WGRAD


def test_pool_spread_gather8():
    W = _ws()
    L = W.lib()
    rng = np.random.default_rng(7)
    nx, ny, nz, c = 8, 6, 4, 16
    x = bf(_rand(rng, nz, ny, nx, c))
    xd = dev(x)
    p = torch.empty((nz // 2, ny // 2, nx // 2, c), dtype=torch.bfloat16, device="cuda")
    assert L.el_nn_pool(nx, ny, nz, c, xd.data_ptr(), p.data_ptr(), None) == 0
    ref = x.reshape(nz // 2, 2, ny // 2, 2, nx // 2, 2, c).mean(dim=(1, 3, 5))
    assert rel_err(p.float().cpu().numpy(), ref.numpy()) < TOL_ACT
    fine = dev(bf(_rand(rng, nz, ny, nx, c)))
    before = fine.float().cpu()
    assert L.el_nn_spread(nx, ny, nz, c, p.data_ptr(), fine.data_ptr(), 0.125, 1, None) == 0
    assert rel_err(fine.float().cpu().numpy(), (before + 0.125 * up2(p.float().cpu())).numpy()) < TOL_ACT
    g = torch.empty_like(p)
    assert L.el_nn_gather8(nx, ny, nz, c, xd.data_ptr(), g.data_ptr(), None) == 0
    assert rel_err(g.float().cpu().numpy(), (ref * 8).numpy()) < TOL_ACT


def test_head_loss_backward_and_adam():
    W = _ws()
    L = W.lib()
    rng = np.random.default_rng(9)
    n = 4096
    d = bf(_rand(rng, n, 16))
    w = torch.from_numpy(_rand(rng, 16)).double()
    b0 = 0.3
    target = torch.from_numpy(_rand(rng, n)).double()
    mask = torch.from_numpy((rng.uniform(size=n) < 0.6).astype(np.uint8))
    dd, wd = dev(d), w.float().cuda()
    bd = torch.tensor([b0], dtype=torch.float32, device="cuda")
    pred = torch.empty(n, dtype=torch.float32, device="cuda")
    assert L.el_nn_head_forward(n, dd.data_ptr(), wd.data_ptr(), bd.data_ptr(), pred.data_ptr(), None) == 0
    ref_pred = d @ w.float().double() + b0
    assert rel_err(pred.cpu().numpy(), ref_pred.numpy()) < 1e-5
    inv_n = 1.0 / float(mask.sum())
    ws = torch.zeros(L.el_nn_head_workspace(n) // 8 + 1, dtype=torch.float64, device="cuda")
    loss = torch.zeros(1, dtype=torch.float64, device="cuda")
    gw = torch.zeros(16, dtype=torch.float32, device="cuda")
    gbias = torch.zeros(1, dtype=torch.float32, device="cuda")
    gd = torch.empty_like(dd)
    tgt, msk = target.float().cuda(), mask.cuda()
    for _ in range(2):  # twice: the workspace's counter must have reset itself
        assert L.el_nn_head_loss_backward(n, dd.data_ptr(), pred.data_ptr(), tgt.data_ptr(), msk.data_ptr(),
                                          wd.data_ptr(), inv_n, gd.data_ptr(), loss.data_ptr(), gw.data_ptr(),
                                          gbias.data_ptr(), ws.data_ptr(), ws.numel() * 8, None) == 0
    torch.cuda.synchronize()
    p_ = pred.double().cpu()
    e = (p_ - target.float().double()) * mask.double()
    assert abs(loss.item() / 2 - float((e * e).sum() * inv_n)) < 1e-6 * max(1.0, loss.item())
    gv = 2 * e * inv_n
    assert rel_err(gw.cpu().numpy() / 2, (gv[:, None] * d).sum(0).numpy()) < 1e-4
    assert abs(gbias.item() / 2 - float(gv.sum())) < 1e-4 * max(1e-3, abs(float(gv.sum())))
    assert rel_err(gd.float().cpu().numpy(), (gv[:, None] * w.float().double()[None, :]).numpy()) < TOL_ACT
    # Adam, two steps, against its formula
    m = 1000
    wp = _rand(rng, m)
    gp = [_rand(rng, m), _rand(rng, m)]
    wt = torch.from_numpy(wp.copy()).cuda()
    mt, vt = torch.zeros_like(wt), torch.zeros_like(wt)
    ref_w, ref_m, ref_v = wp.astype(np.float64), np.zeros(m), np.zeros(m)
    for step in (1, 2):
        gt = torch.from_numpy(gp[step - 1]).cuda()
        assert L.el_nn_adam(m, wt.data_ptr(), gt.data_ptr(), mt.data_ptr(), vt.data_ptr(), 1e-2, 0.9, 0.999, 1e-8,
                            step, None) == 0
        torch.cuda.synchronize()
        assert float(gt.abs().max()) == 0.0
        g64 = gp[step - 1].astype(np.float64)
        ref_m = 0.9 * ref_m + 0.1 * g64
        ref_v = 0.999 * ref_v + 0.001 * g64 * g64
        ref_w = ref_w - 1e-2 * (ref_m / (1 - 0.9 ** step)) / (np.sqrt(ref_v / (1 - 0.999 ** step)) + 1e-8)
    assert rel_err(wt.cpu().numpy(), ref_w) < 1e-5


class _Bf16(torch.autograd.Function):
    """Rounds to bf16 in the forward pass and rounds the gradient to bf16 in the backward pass:
    where the kernels store an activation, and its gradient, as bf16."""

    @staticmethod
    def forward(ctx, t):
        return t.to(torch.bfloat16).to(torch.float64)

    @staticmethod
    def backward(ctx, g):
        return g.to(torch.bfloat16).to(torch.float64)


def _torch_net(W, net, x, bf_round=True):
    """float64 autograd of the same network (bf16-rounded weights), with every activation and
    every activation gradient rounded to bf16 where the kernels store them."""
    params = {}
    acts = {"x": x}

    def rnd(t):
        return _Bf16.apply(t) if bf_round else t

    for name, a_name, up, b_name, cin, cout, level in W.CONVS:
        if a_name in ("p0", "p1", "p2") and a_name not in acts:
            src = {"p0": "e0", "p1": "e1", "p2": "e2"}[a_name]
            s = acts[src]
            z, y, xx, c = s.shape
            acts[a_name] = rnd(s.reshape(z // 2, 2, y // 2, 2, xx // 2, 2, c).mean(dim=(1, 3, 5)))
        wv = net.weight(name).detach().cpu().to(torch.bfloat16).to(torch.float64).reshape(cout, 27, cin)
        bv = net.bias(name).detach().cpu().to(torch.float64)
        wv.requires_grad_(True)
        bv.requires_grad_(True)
        params[name] = (wv, bv)
        inp = acts[a_name]
        if up:
            # the upsampled part's gradient is stored at fine resolution before it is summed
            # down; the skip part's before the pooling path's gradient is added to it
            inp = torch.cat([rnd(up2(inp)), rnd(acts[b_name])], dim=3)
        acts[name] = rnd(torch.relu(conv_ref(inp, wv, bv)))
    hw, hb = net.head()
    hw = hw.detach().cpu().double().requires_grad_(True)
    hb = hb.detach().cpu().double().requires_grad_(True)
    pred = acts["d0"] @ hw + hb
    return pred, params, (hw, hb), acts


def test_network_gradients_match_autograd():
    """The whole network on a 16^3 grid.  Every layer's backward is checked in place against
    float64 autograd fed with the kernels' own stored activations and output gradients (so the
    check is as tight as for a single layer); the end-to-end gradients against an independent
    float64 autograd of the whole network only loosely, because bf16 rounding decisions that go
    the other way multiply through the layers (after 14 layers a quarter of the activations
    differ by an ulp)."""
    W = _ws()
    net = W.WarmStartNet(torch, seed=1)
    n = 16
    rng = np.random.default_rng(11)
    x = net.input_buffer(n, n, n)
    x.zero_()
    xin = bf(_rand(rng, n, n, n, 3))
    x[..., :3].copy_(xin.to(torch.bfloat16).cuda())
    pred = net.forward(n, n, n)
    target = torch.from_numpy(_rand(rng, n, n, n)).cuda()
    fluid = torch.from_numpy((rng.uniform(size=(n, n, n)) < 0.7).astype(np.uint8)).cuda()
    inv_n = 1.0 / float(fluid.sum())
    net.backward(n, n, n, target, fluid, inv_n)
    torch.cuda.synchronize()
    loss = net.take_loss(n, n, n)
    bufs = net._bufs(n, n, n)
    A = {k: v.float().cpu().double() for k, v in bufs["act"].items()}
    G = {k: v.float().cpu().double() for k, v in bufs["grad"].items()}
    # layer by layer, from the kernels' own tensors
    written_once = set()
    for name, a_name, up, b_name, cin, cout, level in W.CONVS:
        if a_name not in ("x", "p0", "p1", "p2", "e0", "e1", "e2"):
            written_once.add(a_name)
    for name, a_name, up, b_name, cin, cout, level in W.CONVS:
        wv = net.weight(name).detach().cpu().to(torch.bfloat16).to(torch.float64).reshape(cout, 27, cin)
        a_ = A[a_name].clone().requires_grad_(True)
        parts = [up2(a_)] if up else [a_]
        if b_name:
            parts.append(A[b_name])
        inp = torch.cat(parts, dim=3) if len(parts) > 1 else parts[0]
        w_ = wv.clone().requires_grad_(True)
        gm = G[name] * (A[name] > 0).double()
        (conv_ref(inp, w_) * gm).sum().backward()
        gw = net.grad_w(name).cpu().numpy().reshape(cout, 27, cin)
        assert rel_err(gw, w_.grad.numpy()) < TOL_WGRAD, (name, rel_err(gw, w_.grad.numpy()))
        assert rel_err(net.grad_b(name).cpu().numpy(), gm.sum(dim=(0, 1, 2)).numpy()) < TOL_WGRAD, name
        if a_name in written_once:
            assert rel_err(G[a_name].numpy(), a_.grad.numpy()) < TOL_ACT, (name, rel_err(G[a_name].numpy(),
                                                                                 a_.grad.numpy()))
    # end to end against an independent float64 network
    xr = torch.zeros((n, n, n, 16), dtype=torch.float64)
    xr[..., :3] = xin
    ref_pred, params, (hw, hb), _ = _torch_net(W, net, xr)
    assert rel_err(pred.cpu().numpy(), ref_pred.detach().numpy()) < 2e-2
    m = fluid.cpu().double()
    e = (ref_pred - target.cpu().double()) * m
    ref_loss = (e * e).sum() * inv_n
    assert abs(loss - ref_loss.item()) < 2e-2 * ref_loss.item()
    ref_loss.backward()
    for name, (wv, bv) in params.items():
        gw = net.grad_w(name).cpu().numpy().reshape(wv.shape)
        assert rel_err(gw, wv.grad.numpy()) < TOL_NET, (name, rel_err(gw, wv.grad.numpy()))
    ghw, ghb = net.head_grads()
    assert rel_err(ghw.cpu().numpy(), hw.grad.numpy()) < 1e-2


TC_PAIRS = [(16, 16), (16, 32), (32, 32), (32, 64), (48, 16), (32, 16), (64, 32), (16, 48), (32, 96)]


@pytest.mark.parametrize("cin,cout", TC_PAIRS)
def test_tcgen05_conv_matches_conv3d_and_mma_sync(cin, cout):
    """The tcgen05 kernel (operands in shared memory, accumulator in TMEM) against torch-CPU conv3d
    and against the mma.sync kernel, on a grid with partial bricks; (48, 16) with the decoder's
    upsampled concatenation, (32, 96) with a ReLU mask as in the backward-data pass."""
    W = _ws()
    L = W.lib()
    assert L.el_nn_tc_supported(cin, cout) == 1
    rng = np.random.default_rng(cin * 7 + cout)
    nx, ny, nz = 20, 34, 4
    w = bf(_rand(rng, cout, 27, cin, scale=(2.0 / (27 * cin)) ** 0.5))
    bias = torch.from_numpy(_rand(rng, cout, scale=0.1))
    fwd, _ = _pack(L, w.numpy(), cin, cout)
    nb = L.el_nn_packed_weight_bytes(cin, cout) // 2
    tcw = torch.empty(nb, dtype=torch.bfloat16, device="cuda")
    wd = torch.from_numpy(np.asarray(w.numpy(), np.float32)).cuda()
    assert L.el_nn_pack_weights_tc(cin, cout, wd.data_ptr(), tcw.data_ptr(), None, None) == 0
    mask = None
    if cin == 48:
        a = bf(_rand(rng, nz // 2, ny // 2, nx // 2, 32))
        b = bf(_rand(rng, nz, ny, nx, 16))
        inp = torch.cat([up2(a), b], dim=3)
        args_in = (dev(a), 32, 1, dev(b), 16)
    else:
        x = bf(_rand(rng, nz, ny, nx, cin))
        inp = x
        args_in = (dev(x), cin, 0, None, 0)
        if cin == 32 and cout == 96:
            m = bf(_rand(rng, nz, ny, nx, cin))
            mask = dev(m)
            inp = x * (m > 0).double()
    ref = torch.relu(conv_ref(inp, w, bias.double()))
    outs = []
    for use_tc in (True, False):
        out = torch.empty((nz, ny, nx, cout), dtype=torch.bfloat16, device="cuda")
        bd = bias.cuda()
        args = _args(W, (nx, ny, nz), cin, cout, args_in[0], args_in[1], args_in[2], args_in[3], args_in[4])
        args.weights, args.bias, args.relu = fwd.data_ptr(), bd.data_ptr(), 1
        if mask is not None:
            args.mask = mask.data_ptr()
        args.out_a, args.out_a_channels = out.data_ptr(), cout
        if use_tc:
            args.weights_tc = tcw.data_ptr()
        assert L.el_nn_conv3_forward(C.byref(args), None) == 0
        torch.cuda.synchronize()
        outs.append(out.float().cpu().numpy())
    assert L.el_nn_take_error() == 0
    assert rel_err(outs[0], ref.numpy()) < TOL_ACT, rel_err(outs[0], ref.numpy())
    assert rel_err(outs[0], outs[1]) < TOL_ACT
