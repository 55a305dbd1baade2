"""Learned warm start for the pressure solve: network, data recorder, training and evaluation.

A 3D convolutional encoder-decoder (4 levels, 16/32/64/64 channels, 3x3x3 kernels, ReLU,
2x2x2 average pooling down, nearest upsampling and skip concatenation up, a 1x1x1 head) maps
the scene's (level set, divergence, solid mask) to a pressure guess.  Every tensor operation
runs in the library's own CUDA kernels through the C ABI (BF16 tensor-core implicit-GEMM
convolutions with FP32 accumulation, forward and backward, Adam); PyTorch only owns the device
memory here.  The guess is refined by el_solve_pressure(initial_guess=1) to the same tolerance
as a solve from zero, so the network can only change how many iterations that takes.

Layout (channels-last bf16, one sample): level l has grid (nx, ny, nz) / 2^l.

    x (16 ch: phi, b, solid, 0...)
    e0a, e0  = conv 16->16, 16->16           level 0   (e0: skip)
    e1a, e1  = conv 16->32, 32->32 of pool(e0) level 1 (e1: skip)
    e2a, e2  = conv 32->64, 64->64 of pool(e1) level 2 (e2: skip)
    b0, b1   = conv 64->64, 64->64 of pool(e2) level 3
    d2a, d2  = conv [up(b1), e2] 128->64, 64->64
    d1a, d1  = conv [up(d2), e1]  96->32, 32->32
    d0a, d0  = conv [up(d1), e0]  48->16, 16->16
    pred     = head 16->1 (FP32)

Training targets are the solver's own converged pressures, recorded from simulated scenes
(``record``), in the scaling of el_warmstart_features.  The loss is the guess's error in the
solver's energy norm, e . A e / t . A t -- what conjugate gradients minimises, so the network is
pushed towards errors the solver removes cheaply -- or, optionally, the mean square error over
fluid cells.
"""

import ctypes as C
import math
import time

import numpy as np

from . import EL_OK, ELError, load, status_string

FEAT = 16

# name, input a, upsample a, input b (skip), cin, cout, level
CONVS = [
    ("e0a", "x", 0, None, 16, 16, 0),
    ("e0", "e0a", 0, None, 16, 16, 0),
    ("e1a", "p0", 0, None, 16, 32, 1),
    ("e1", "e1a", 0, None, 32, 32, 1),
    ("e2a", "p1", 0, None, 32, 64, 2),
    ("e2", "e2a", 0, None, 64, 64, 2),
    ("b0", "p2", 0, None, 64, 64, 3),
    ("b1", "b0", 0, None, 64, 64, 3),
    ("d2a", "b1", 1, "e2", 128, 64, 2),
    ("d2", "d2a", 0, None, 64, 64, 2),
    ("d1a", "d2", 1, "e1", 96, 32, 1),
    ("d1", "d1a", 0, None, 32, 32, 1),
    ("d0a", "d1", 1, "e0", 48, 16, 0),
    ("d0", "d0a", 0, None, 16, 16, 0),
]
POOLS = [("p0", "e0", 0, 16), ("p1", "e1", 1, 32), ("p2", "e2", 2, 64)]  # name, source, source level, channels
CHANNELS = {"x": 16, "p0": 16, "p1": 32, "p2": 64, **{c[0]: c[5] for c in CONVS}}
LEVEL = {"x": 0, "p0": 1, "p1": 2, "p2": 3, **{c[0]: c[6] for c in CONVS}}


class ConvArgs(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("cin", C.c_int), ("cout", C.c_int),
                ("in_a", C.c_void_p), ("ca", C.c_int), ("upsample_a", C.c_int), ("in_b", C.c_void_p),
                ("cb", C.c_int), ("mask", C.c_void_p), ("weights", C.c_void_p), ("bias", C.c_void_p),
                ("relu", C.c_int), ("out_a", C.c_void_p), ("out_a_channels", C.c_int), ("out_b", C.c_void_p),
                ("weights_tc", C.c_void_p)]


_declared = False


def lib():
    global _declared
    L = load()
    if not _declared:
        vp, i, sz, f, d, i64 = C.c_void_p, C.c_int, C.c_size_t, C.c_float, C.c_double, C.c_int64
        L.el_nn_conv3_forward.argtypes = [C.POINTER(ConvArgs), vp]
        L.el_nn_conv3_backward_weight_workspace.argtypes = [i, i, i, i, i]
        L.el_nn_conv3_backward_weight_workspace.restype = sz
        L.el_nn_conv3_backward_weight.argtypes = [C.POINTER(ConvArgs), vp, vp, vp, vp, sz, vp]
        L.el_nn_packed_weight_bytes.argtypes = [i, i]
        L.el_nn_packed_weight_bytes.restype = sz
        L.el_nn_pack_weights.argtypes = [i, i, vp, vp, vp, vp]
        L.el_nn_pack_weights_tc.argtypes = [i, i, vp, vp, vp, vp]
        L.el_nn_tc_supported.argtypes = [i, i]
        L.el_nn_tc_preferred.argtypes = [i, i]
        L.el_nn_take_error.argtypes = []
        L.el_nn_pool.argtypes = [i, i, i, i, vp, vp, vp]
        L.el_nn_spread.argtypes = [i, i, i, i, vp, vp, f, i, vp]
        L.el_nn_gather8.argtypes = [i, i, i, i, vp, vp, vp]
        L.el_nn_head_forward.argtypes = [i64, vp, vp, vp, vp, vp]
        L.el_nn_head_workspace.argtypes = [i64]
        L.el_nn_head_workspace.restype = sz
        L.el_nn_head_loss_backward.argtypes = [i64, vp, vp, vp, vp, vp, d, vp, vp, vp, vp, vp, sz, vp]
        L.el_nn_head_energy_loss_backward.argtypes = [i, i, i, vp, vp, vp, vp, vp, vp, d, vp, vp, vp, vp, vp, sz,
                                                      vp]
        L.el_nn_adam.argtypes = [i64, vp, vp, vp, vp, f, f, f, f, i, vp]
        L.el_warmstart_features.argtypes = [vp, i, d, vp, vp, vp, vp, vp]
        L.el_warmstart_set_guess.argtypes = [vp, vp]
        _declared = True
    return L


def _ok(st, what):
    if st != EL_OK:
        raise ELError(st, f"{what}: {status_string(st)}")


def _p(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


class WarmStartNet:
    """The network's parameters (FP32 masters, Adam moments, packed bf16 copies) and, per grid
    size, its activation and gradient buffers."""

    def __init__(self, torch, device="cuda", seed=0, lr=1e-3, tensor_cores="auto"):
        """tensor_cores: "auto" runs the tcgen05 kernel on the layers where it is the faster one,
        True on every layer it supports, False never."""
        self.torch = torch
        self.tensor_cores = tensor_cores
        self.dev = torch.device(device)
        self.L = lib()
        self.lr = lr
        self.step_count = 0
        rng = np.random.default_rng(seed)
        # one flat FP32 buffer for all parameters (and one each for grads and Adam moments)
        self.offsets = {}
        sizes = []
        off = 0
        for name, _, _, _, cin, cout, _ in CONVS:
            self.offsets[name] = (off, off + 27 * cin * cout)  # weights, then bias
            off += 27 * cin * cout + cout
            sizes.append((name, cin, cout))
        self.offsets["head"] = (off, off + FEAT)
        off += FEAT + 1
        self.nparams = off
        init = np.zeros(off, np.float32)
        for name, cin, cout in sizes:
            w0, b0 = self.offsets[name]
            # He initialisation for ReLU: std = sqrt(2 / fan_in)
            init[w0:b0] = rng.normal(0.0, math.sqrt(2.0 / (27 * cin)), 27 * cin * cout).astype(np.float32)
        h0, hb = self.offsets["head"]
        init[h0:hb] = rng.normal(0.0, math.sqrt(1.0 / FEAT), FEAT).astype(np.float32)
        self.params = torch.from_numpy(init).to(self.dev)
        self.grads = torch.zeros_like(self.params)
        self.m = torch.zeros_like(self.params)
        self.v = torch.zeros_like(self.params)
        self.packed = {}
        self.packed_tc = {}  # forward / backward-data weights for the tcgen05 kernel, where it applies
        for name, cin, cout in sizes:
            nb = self.L.el_nn_packed_weight_bytes(cin, cout) // 2
            self.packed[name] = (torch.empty(nb, dtype=torch.bfloat16, device=self.dev),
                                 torch.empty(nb, dtype=torch.bfloat16, device=self.dev))
            pick = self.L.el_nn_tc_preferred if tensor_cores == "auto" else self.L.el_nn_tc_supported
            fwd_tc, bwd_tc = pick(cin, cout), pick(cout, cin)
            if tensor_cores and (fwd_tc or bwd_tc):
                self.packed_tc[name] = (torch.empty(nb, dtype=torch.bfloat16, device=self.dev) if fwd_tc else None,
                                        torch.empty(nb, dtype=torch.bfloat16, device=self.dev) if bwd_tc else None)
        self.buffers = {}
        self.pack()

    # -- parameters ----------------------------------------------------------------------
    def stream(self):
        return C.c_void_p(self.torch.cuda.current_stream(self.dev).cuda_stream)

    def weight(self, name):
        w0, b0 = self.offsets[name]
        return self.params[w0:b0]

    def bias(self, name):
        _, b0 = self.offsets[name]
        cout = [c[5] for c in CONVS if c[0] == name][0]
        return self.params[b0:b0 + cout]

    def grad_w(self, name):
        w0, b0 = self.offsets[name]
        return self.grads[w0:b0]

    def grad_b(self, name):
        _, b0 = self.offsets[name]
        cout = [c[5] for c in CONVS if c[0] == name][0]
        return self.grads[b0:b0 + cout]

    def head(self):
        h0, hb = self.offsets["head"]
        return self.params[h0:hb], self.params[hb:hb + 1]

    def head_grads(self):
        h0, hb = self.offsets["head"]
        return self.grads[h0:hb], self.grads[hb:hb + 1]

    def pack(self):
        s = self.stream()
        for name, _, _, _, cin, cout, _ in CONVS:
            fwd, bwd = self.packed[name]
            _ok(self.L.el_nn_pack_weights(cin, cout, _p(self.weight(name)), _p(fwd), _p(bwd), s), "pack_weights")
            if name in self.packed_tc:
                tf, tb = self.packed_tc[name]
                scratch = tf if tf is not None else self._scratch(tb)
                _ok(self.L.el_nn_pack_weights_tc(cin, cout, _p(self.weight(name)), _p(scratch), _p(tb), s),
                    "pack_weights_tc")

    def _scratch(self, like):
        if getattr(self, "_pack_scratch", None) is None or self._pack_scratch.numel() < like.numel():
            self._pack_scratch = self.torch.empty_like(like)
        return self._pack_scratch

    def state_dict(self):
        return {"params": self.params.detach().cpu().numpy().copy(), "step": self.step_count}

    def load_state_dict(self, d):
        self.params.copy_(self.torch.from_numpy(d["params"]).to(self.dev))
        self.step_count = int(d.get("step", 0))
        self.pack()

    # -- buffers per grid ------------------------------------------------------------------
    def _bufs(self, nx, ny, nz):
        key = (nx, ny, nz)
        if key in self.buffers:
            return self.buffers[key]
        if nx % 8 or ny % 8 or nz % 8:
            raise ValueError("grid sizes must be multiples of 8 (three 2x2x2 poolings)")
        torch = self.torch
        dims = [(nx >> l, ny >> l, nz >> l) for l in range(4)]

        def act(name):
            x, y, z = dims[LEVEL[name]]
            return torch.empty((z, y, x, CHANNELS[name]), dtype=torch.bfloat16, device=self.dev)

        names = ["x"] + [c[0] for c in CONVS] + [p[0] for p in POOLS]
        b = {"dims": dims, "act": {n: act(n) for n in names}, "grad": {n: act(n) for n in names if n != "x"}}
        # fine-resolution gradient of an upsampled input (largest: d2a's 64 channels at level 2 etc.)
        b["gup"] = {c[0]: torch.empty((dims[c[6]][2], dims[c[6]][1], dims[c[6]][0], CHANNELS[c[1]]),
                                      dtype=torch.bfloat16, device=self.dev) for c in CONVS if c[2]}
        n = nx * ny * nz
        b["pred"] = torch.empty((nz, ny, nx), dtype=torch.float32, device=self.dev)
        ws = max(self.L.el_nn_conv3_backward_weight_workspace(*dims[c[6]], c[4], c[5]) for c in CONVS)
        b["ws"] = torch.empty(ws // 4 + 1, dtype=torch.float32, device=self.dev)
        hw = self.L.el_nn_head_workspace(n)
        b["head_ws"] = torch.zeros(hw // 8 + 1, dtype=torch.float64, device=self.dev)
        b["loss"] = torch.zeros(1, dtype=torch.float64, device=self.dev)
        self.buffers[key] = b
        return b

    def input_buffer(self, nx, ny, nz):
        return self._bufs(nx, ny, nz)["act"]["x"]

    # -- passes ------------------------------------------------------------------------------
    def _conv_args(self, b, name, a_name, up, b_name, cin, cout, level):
        nx, ny, nz = b["dims"][level]
        A = b["act"]
        a = ConvArgs()
        a.nx, a.ny, a.nz, a.cin, a.cout = nx, ny, nz, cin, cout
        a.in_a = A[a_name].data_ptr()
        a.ca = CHANNELS[a_name]
        a.upsample_a = up
        a.in_b = A[b_name].data_ptr() if b_name else None
        a.cb = CHANNELS[b_name] if b_name else 0
        return a

    def forward(self, nx, ny, nz):
        """pred = net(x) with x = input_buffer(nx, ny, nz) filled by the caller."""
        b = self._bufs(nx, ny, nz)
        A = b["act"]
        s = self.stream()
        for name, a_name, up, b_name, cin, cout, level in CONVS:
            if name == "e1a":
                self._pool(b, 0, s)
            elif name == "e2a":
                self._pool(b, 1, s)
            elif name == "b0":
                self._pool(b, 2, s)
            args = self._conv_args(b, name, a_name, up, b_name, cin, cout, level)
            args.weights = self.packed[name][0].data_ptr()
            if name in self.packed_tc and self.packed_tc[name][0] is not None:
                args.weights_tc = self.packed_tc[name][0].data_ptr()
            args.bias = self.bias(name).data_ptr()
            args.relu = 1
            args.out_a = A[name].data_ptr()
            args.out_a_channels = cout
            args.out_b = None
            _ok(self.L.el_nn_conv3_forward(C.byref(args), s), f"conv {name}")
        hw, hb = self.head()
        _ok(self.L.el_nn_head_forward(nx * ny * nz, _p(A["d0"]), _p(hw), _p(hb), _p(b["pred"]), s), "head")
        return b["pred"]

    def _pool(self, b, i, s):
        name, src, lvl, c = POOLS[i]
        nx, ny, nz = b["dims"][lvl]
        _ok(self.L.el_nn_pool(nx, ny, nz, c, _p(b["act"][src]), _p(b["act"][name]), s), "pool")

    def backward(self, nx, ny, nz, target, fluid, inv_n, couplings=None):
        """Accumulates the gradients of the loss of the last forward -- the energy norm
        e . A^ e when the scaled operator's couplings are given, else the mean square error over
        the fluid cells -- times inv_n, and adds the loss to the accumulator (take_loss)."""
        b = self._bufs(nx, ny, nz)
        A, G = b["act"], b["grad"]
        s = self.stream()
        hw, _ = self.head()
        gw, gb = self.head_grads()
        ws = b["head_ws"]
        if couplings is not None:
            _ok(self.L.el_nn_head_energy_loss_backward(nx, ny, nz, _p(A["d0"]), _p(b["pred"]), _p(target),
                                                       _p(couplings), _p(fluid), _p(hw), inv_n, _p(G["d0"]), _p(b["loss"]),
                                                       _p(gw), _p(gb), _p(ws), ws.numel() * 8, s), "energy loss")
        else:
            _ok(self.L.el_nn_head_loss_backward(nx * ny * nz, _p(A["d0"]), _p(b["pred"]), _p(target), _p(fluid),
                                                _p(hw), inv_n, _p(G["d0"]), _p(b["loss"]), _p(gw), _p(gb), _p(ws),
                                                ws.numel() * 8, s), "head backward")
        wsp = b["ws"]
        for name, a_name, up, b_name, cin, cout, level in reversed(CONVS):
            args = self._conv_args(b, name, a_name, up, b_name, cin, cout, level)
            args.out_a = A[name].data_ptr()  # the forward output: ReLU' mask
            _ok(self.L.el_nn_conv3_backward_weight(C.byref(args), _p(G[name]), _p(self.grad_w(name)),
                                                   _p(self.grad_b(name)), _p(wsp), wsp.numel() * 4, s),
                f"wgrad {name}")
            if name == "e0a":
                continue  # no gradient for the network input
            nxl, nyl, nzl = b["dims"][level]
            d = ConvArgs()
            d.nx, d.ny, d.nz = nxl, nyl, nzl
            d.cin, d.cout = cout, cin
            d.in_a, d.ca, d.upsample_a = G[name].data_ptr(), cout, 0
            d.in_b, d.cb = None, 0
            d.mask = A[name].data_ptr()
            d.weights = self.packed[name][1].data_ptr()
            if name in self.packed_tc and self.packed_tc[name][1] is not None:
                d.weights_tc = self.packed_tc[name][1].data_ptr()
            d.bias, d.relu = None, 0
            if up:
                d.out_a, d.out_a_channels, d.out_b = b["gup"][name].data_ptr(), CHANNELS[a_name], G[b_name].data_ptr()
            else:
                d.out_a, d.out_a_channels, d.out_b = G[a_name].data_ptr(), cin, None
            _ok(self.L.el_nn_conv3_forward(C.byref(d), s), f"dgrad {name}")
            if up:
                _ok(self.L.el_nn_gather8(nxl, nyl, nzl, CHANNELS[a_name], _p(b["gup"][name]), _p(G[a_name]), s),
                    "gather8")
            if a_name in ("p0", "p1", "p2"):
                pname, src, lvl, c = [p for p in POOLS if p[0] == a_name][0]
                fx, fy, fz = b["dims"][lvl]
                _ok(self.L.el_nn_spread(fx, fy, fz, c, _p(G[a_name]), _p(G[src]), 0.125, 1, s), "pool backward")

    def take_loss(self, nx, ny, nz):
        b = self._bufs(nx, ny, nz)
        v = float(b["loss"].item())
        b["loss"].zero_()
        return v

    def adam_step(self, lr=None, beta1=0.9, beta2=0.999, eps=1e-8):
        self.step_count += 1
        _ok(self.L.el_nn_adam(self.nparams, _p(self.params), _p(self.grads), _p(self.m), _p(self.v),
                              lr or self.lr, beta1, beta2, eps, self.step_count, self.stream()), "adam")
        self.pack()


# ---- data: recorded solves ------------------------------------------------------------------

class Dataset:
    """Recorded tuples on the device: features (the 4 leading channels phi, b, solid, 0 -- the
    rest of the network input is zero), the scaled operator's couplings (4 bf16 per cell), the
    target pressure, the fluid mask; per tuple on the host, the fluid cell count and the
    target's energy."""

    def __init__(self, torch, shape, capacity, device="cuda"):
        nx, ny, nz = shape
        self.shape = shape
        self.torch = torch
        self.x = torch.empty((capacity, nz, ny, nx, 4), dtype=torch.bfloat16, device=device)
        self.c = torch.empty((capacity, nz, ny, nx, 4), dtype=torch.bfloat16, device=device)
        self.t = torch.empty((capacity, nz, ny, nx), dtype=torch.float32, device=device)
        self.f = torch.empty((capacity, nz, ny, nx), dtype=torch.uint8, device=device)
        self.count = np.zeros(capacity)
        self.energy = np.zeros(capacity)
        self.n = 0

    def __len__(self):
        return self.n


def record(el, torch, specs, steps_per_scene, shape, params, cfl=1.0, frame=1.0 / 60.0, capacity=None,
           dtype=None):
    """Simulate each scene spec (resized to `shape`) and record one tuple after every step:
    the network input of the system that step solved and the converged pressure."""
    nx, ny, nz = shape
    cap = capacity or len(specs) * steps_per_scene
    ds = Dataset(torch, shape, cap)
    L = lib()
    feat = torch.zeros((nz, ny, nx, FEAT), dtype=torch.bfloat16, device="cuda")
    for spec in specs:
        if ds.n >= cap:
            break
        sim = el.Simulator(nx, ny, nz, dtype=dtype if dtype is not None else el.EL_F32)
        sim.set_stream(torch.cuda.current_stream().cuda_stream)
        sim.init_scene(dict(spec, shape=shape))
        for _ in range(steps_per_scene):
            if ds.n >= cap:
                break
            dt = min(sim.calc_time_step(cfl), frame)
            st = sim.step(dt, params)
            if st["status"] != EL_OK:
                continue
            i = ds.n
            scales = (C.c_double * 3)()  # (asking for them also waits for the scene's stream)
            _ok(L.el_warmstart_features(sim.h, 0, 0.0, _p(feat), _p(ds.c[i]), _p(ds.t[i]), _p(ds.f[i]), scales),
                "features")
            if not scales[2] > 0:
                continue  # no pressure to learn (a system at rest)
            ds.x[i].copy_(feat[..., :4])
            ds.count[i] = st["fluid_cells"]
            ds.energy[i] = scales[2]
            ds.n += 1
        torch.cuda.synchronize()
        sim.close()
    return ds


def train(net, ds, epochs=1, batch=4, lr=None, seed=0, log=None, max_steps=None, loss="energy"):
    """Adam, `batch` tuples per update (gradients accumulated).  loss="energy": the error in the
    solver's energy norm relative to the target's, e . A^ e / t . A^ t; "mse": mean square error
    over the fluid cells."""
    torch = net.torch
    nx, ny, nz = ds.shape
    x = net.input_buffer(nx, ny, nz)
    x.zero_()
    rng = np.random.default_rng(seed)
    history = []
    steps = 0
    t0 = time.perf_counter()
    for ep in range(epochs):
        order = rng.permutation(ds.n)
        for s0 in range(0, ds.n, batch):
            idx = order[s0:s0 + batch]
            for i in idx:
                x[..., :4].copy_(ds.x[i])
                net.forward(nx, ny, nz)
                if loss == "energy":
                    net.backward(nx, ny, nz, ds.t[i], ds.f[i], 1.0 / (ds.energy[i] * len(idx)), couplings=ds.c[i])
                else:
                    net.backward(nx, ny, nz, ds.t[i], ds.f[i], 1.0 / (max(1.0, float(ds.count[i])) * len(idx)))
            net.adam_step(lr)
            steps += 1
            if log is not None and (steps % log == 0):
                history.append((steps, net.take_loss(nx, ny, nz) / 1.0))
            if max_steps and steps >= max_steps:
                break
        if max_steps and steps >= max_steps:
            break
    torch.cuda.synchronize()
    return {"steps": steps, "seconds": time.perf_counter() - t0, "history": history}


def predict_guess(net, sim, dt):
    """Build the scene's system for dt, run the network, write the scaled guess into the
    pressure field (ready for solve_pressure(initial_guess=1))."""
    L = lib()
    torch = net.torch
    x = net.input_buffer(sim.ni, sim.nj, sim.nk)
    torch.cuda.current_stream().synchronize()  # the input buffer is free
    sim._check(L.el_warmstart_features(sim.h, 1, dt, _p(x), None, None, None, None), "warmstart_features")
    sim._check(sim.lib.el_ctx_sync(sim.h), "sync")  # features written (the scene's stream)
    pred = net.forward(sim.ni, sim.nj, sim.nk)
    torch.cuda.current_stream().synchronize()  # prediction written (the network's stream)
    sim._check(L.el_warmstart_set_guess(sim.h, _p(pred)), "warmstart_set_guess")
    return pred
