"""Surrogate tensor-core kernels against the float64 CPU oracle, and training (GPU)."""
import ctypes as C

import numpy as np
import pytest

from conftest import module

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import sg_oracle as SO  # noqa: E402


@pytest.fixture(scope="module")
def sg():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import __graft_entry__
    __graft_entry__.build()
    return module("surrogate")


def _bf(t):
    return t.to(torch.bfloat16)


def _rel(a, b):
    return ((a - b).norm() / b.norm()).item()


@pytest.mark.parametrize("cin,cout", [(16, 32), (32, 32)])
def test_conv_forward_matches_oracle(sg, cin, cout):
    n = 32
    g = torch.Generator().manual_seed(cin + cout)
    x = torch.randn((n, n, n, cin), generator=g)
    w = torch.randn((27, cout, cin), generator=g) * 0.1
    b = torch.randn(cout, generator=g) * 0.1
    xb, wb = _bf(x), _bf(w)
    ref = torch.relu(SO.conv3d(xb.double(), wb.double(), b.double()))
    net = sg.SurrogateNet()
    out = torch.empty((n, n, n, cout), dtype=torch.bfloat16, device="cuda")
    net._conv(n, cin, cout, 0, xb.cuda(), wb.cuda(), b.cuda(), out)
    got = out.float().cpu().double()
    assert _rel(got, ref) < 4e-3                       # bf16 rounding of the output


def test_input_gradient_matches_oracle(sg):
    n, cin, cout = 32, 32, 32
    g = torch.Generator().manual_seed(3)
    xin = torch.relu(torch.randn((n, n, n, cin), generator=g))       # layer input (ReLU output)
    w = torch.randn((27, cout, cin), generator=g) * 0.1
    dz = torch.randn((n, n, n, cout), generator=g)
    wb, dzb, xb = _bf(w), _bf(dz), _bf(xin)
    x64 = xb.double().requires_grad_(True)
    y = SO.conv3d(x64, wb.double())
    y.backward(dzb.double())
    ref = x64.grad * (xb.double() > 0)
    net = sg.SurrogateNet()
    wflip = wb.float().flip(0).transpose(1, 2).contiguous().to(torch.bfloat16)
    out = torch.empty((n, n, n, cin), dtype=torch.bfloat16, device="cuda")
    net._conv(n, cout, cin, 2, dzb.cuda(), wflip.cuda(), None, out, mask=xb.cuda())
    assert _rel(out.float().cpu().double(), ref) < 4e-3


@pytest.mark.parametrize("cin,cout", [(16, 32), (32, 32), (32, 16)])
def test_weight_gradient_matches_oracle(sg, cin, cout):
    n = 32
    g = torch.Generator().manual_seed(7 + cin)
    x = torch.randn((n, n, n, cin), generator=g)
    dz = torch.randn((n, n, n, cout), generator=g)
    xb, dzb = _bf(x), _bf(dz)
    w64 = torch.zeros((27, cout, cin), dtype=torch.float64, requires_grad=True)
    b64 = torch.zeros(cout, dtype=torch.float64, requires_grad=True)
    SO.conv3d(xb.double(), w64, b64).backward(dzb.double())
    net = sg.SurrogateNet()
    dw = torch.empty((27, cout, cin), device="cuda")
    db = torch.empty(cout, device="cuda")
    net._wgrad(n, cin, cout, xb.cuda(), dzb.cuda(), dw, db)
    assert _rel(dw.cpu().double(), w64.grad) < 1e-5   # fp32 sums of exact bf16 products
    assert _rel(db.cpu().double(), b64.grad) < 1e-5


def test_network_gradients_match_float64_autograd(sg):
    n = 16
    net = sg.SurrogateNet(seed=1)
    g = torch.Generator(device="cuda").manual_seed(5)
    delta = torch.randn((n, n, n), device="cuda", generator=g) * 0.3
    target = (torch.rand((n, n, n), device="cuda", generator=g) > 0.5).float()
    f = sg.features(delta, 8.0, 30.0, 15.0, 2e4)
    pred, acts = net.forward(f, keep=True)
    dws, dbs = net.backward(acts, pred, target)
    ws = [w.to(torch.bfloat16).double().cpu() for w in net.w]
    rdw, rdb, rpred = SO.net_grads(f.double().cpu(), ws, [b.cpu() for b in net.b], target.cpu())
    assert _rel(pred.cpu().double(), rpred) < 2e-2
    for li, (a, r) in enumerate(zip(dws, rdw)):
        cos = torch.nn.functional.cosine_similarity(a.cpu().double().flatten(), r.flatten(), dim=0).item()
        assert cos > 0.98, (li, cos)


TC_CASES = [(16, 32, 0), (32, 32, 0), (32, 16, 1), (32, 32, 2), (16, 32, 2)]


@pytest.mark.parametrize("cin,cout,mode", TC_CASES)
def test_tcgen05_conv_matches_oracle_and_mma_sync(sg, cin, cout, mode):
    # 128^3 runs on the tcgen05/TMEM kernels; the same call with the mma.sync kernels selected and
    # the float64 oracle on four z-planes (both x edges, both z edges) must agree
    n = 128
    lib = sg._lib.load()
    g = torch.Generator().manual_seed(100 + cin + cout + mode)
    x = _bf(torch.randn((n, n, n, cin), generator=g))
    w = _bf(torch.randn((27, cout, cin), generator=g) * 0.1)
    b = None if mode == 2 else torch.randn(cout, generator=g) * 0.1
    mask = _bf(torch.relu(torch.randn((n, n, n, cout), generator=g))) if mode == 2 else None
    shape, dt = ((n, n, n), torch.float32) if mode == 1 else ((n, n, n, cout), torch.bfloat16)
    net = sg.SurrogateNet()
    xd, wd = x.cuda(), w.cuda()
    bd = b.cuda() if b is not None else None
    md = mask.cuda() if mask is not None else None
    assert lib.sg_conv3d_get_impl() == 0
    out_tc = torch.empty(shape, dtype=dt, device="cuda")
    net._conv(n, cin, cout, mode, xd, wd, bd, out_tc, md)
    assert lib.sg_check() == 0
    out_ms = torch.empty(shape, dtype=dt, device="cuda")
    assert lib.sg_conv3d_set_impl(1) == 0
    try:
        net._conv(n, cin, cout, mode, xd, wd, bd, out_ms, md)
    finally:
        lib.sg_conv3d_set_impl(0)
    assert _rel(out_tc.float(), out_ms.float()) < 2e-3   # same products, other summation order
    planes = [0, 1, 63, 127]
    ref = SO.conv3d_planes(x.double(), w.double(), b, planes)
    if mode == 0:
        ref = torch.relu(ref)
    elif mode == 1:
        ref = torch.sigmoid(ref[..., 0])
    else:
        ref = ref * (mask[planes].double() > 0)
    got = out_tc[planes].cpu().double()
    assert _rel(got, ref) < 4e-3                       # bf16 rounding of the output
    if mode != 1:
        assert torch.isfinite(out_tc.float()).all()


@pytest.mark.parametrize("cin,cout", [(16, 32), (32, 32), (32, 16)])
def test_tcgen05_weight_gradient_matches_oracle_and_mma_sync(sg, cin, cout):
    # 128^3: the tcgen05/TMEM weight gradient (MN-major operands, the ones row for the bias) against
    # the mma.sync kernel on every tap, and against float64 sums on three taps and the bias
    n = 128
    lib = sg._lib.load()
    g = torch.Generator().manual_seed(300 + cin + cout)
    xb = _bf(torch.randn((n, n, n, cin), generator=g))
    dzb = _bf(torch.randn((n, n, n, cout), generator=g))
    net = sg.SurrogateNet()
    res = []
    for impl in (0, 1):
        dw = torch.empty((27, cout, cin), device="cuda")
        db = torch.empty(cout, device="cuda")
        assert lib.sg_conv3d_set_impl(impl) == 0
        try:
            net._wgrad(n, cin, cout, xb.cuda(), dzb.cuda(), dw, db)
            net._wgrad(n, cin, cout, xb.cuda(), dzb.cuda(), dw, db)     # twice: accumulators restart
        finally:
            lib.sg_conv3d_set_impl(0)
        res.append((dw.cpu().double(), db.cpu().double()))
    assert lib.sg_check() == 0
    (dw_tc, db_tc), (dw_ms, db_ms) = res
    assert _rel(dw_tc, dw_ms) < 1e-4 and _rel(db_tc, db_ms) < 1e-4     # fp32 sums, other orders
    x64 = xb.double().numpy().reshape(-1, cin)
    dz64 = dzb.double().numpy().reshape(-1, cout)
    assert np.allclose(db_tc.numpy(), dz64.sum(0), rtol=1e-4, atol=1e-2)
    xs = xb.double().numpy()
    for t in (13, 0, 26):                               # (0,0,0), (-1,-1,-1), (+1,+1,+1)
        dz_, dy_, dx_ = t // 9 - 1, (t // 3) % 3 - 1, t % 3 - 1
        shifted = np.roll(xs, shift=(-dz_, -dy_, -dx_), axis=(0, 1, 2)).reshape(-1, cin)
        ref = dz64.T @ shifted                           # [cout, cin]
        err = np.abs(dw_tc[t].numpy() - ref).max() / np.abs(ref).max()
        assert err < 1e-4, (t, err)


def test_tcgen05_network_step_matches_mma_sync(sg):
    # one forward + backward of the full network at 128^3 on both kernel families
    n = 128
    lib = sg._lib.load()
    net = sg.SurrogateNet(seed=2)
    g = torch.Generator(device="cuda").manual_seed(9)
    delta = torch.randn((n, n, n), device="cuda", generator=g) * 0.5
    target = (torch.rand((n, n, n), device="cuda", generator=g) > 0.5).float()
    f = sg.features(delta, 7.0, 40.0, 20.0, 3e4)
    res = []
    for impl in (0, 1):
        assert lib.sg_conv3d_set_impl(impl) == 0
        try:
            pred, acts = net.forward(f, keep=True)
            dws, dbs = net.backward(acts, pred, target)
        finally:
            lib.sg_conv3d_set_impl(0)
        res.append((pred, dws))
    assert lib.sg_check() == 0
    assert _rel(res[0][0], res[1][0]) < 1e-2
    for li, (a, c) in enumerate(zip(res[0][1], res[1][1])):
        cos = torch.nn.functional.cosine_similarity(a.flatten().double(), c.flatten().double(), dim=0).item()
        assert cos > 0.99, (li, cos)


def test_training_beats_the_untrained_network(sg):
    # engine-generated pairs at 32^3; the trained surrogate must beat its own initialisation and
    # the constant (mean x_HI) predictor on held-out realisations
    gen = sg.DataGenerator(n=32, box_len=50.0)
    rng = np.random.default_rng(0)
    train = [gen.sample(1000 + i, sg.draw_params(rng)) for i in range(48)]
    held = [gen.sample(5000 + i, sg.draw_params(rng)) for i in range(8)]
    net = sg.SurrogateNet(seed=0)
    before = sg.evaluate(net, held)["mean_abs_dxHI"]
    losses = sg.train(net, train, epochs=6, lr=3e-4)
    after = sg.evaluate(net, held)["mean_abs_dxHI"]
    mean_pred = np.mean([s.xH.mean().item() for s in train])
    const = np.mean([(s.xH - mean_pred).abs().mean().item() for s in held])
    assert np.isfinite(losses).all()
    assert losses[-len(train):].mean() < losses[:len(train)].mean()
    assert after < before, (after, before)
    assert after < 0.6 * const, (after, const)


def test_sweep_uses_the_engine_as_fallback_and_judge(sg):
    gen = sg.DataGenerator(n=32, box_len=50.0)
    net = sg.SurrogateNet(seed=0)
    rng = np.random.default_rng(3)
    pts = [sg.draw_params(rng) for _ in range(4)]
    deltas = [gen.density(200 + i, p["z"]) for i, p in enumerate(pts)]
    # a budget nothing can miss: every point is served by the surrogate, every one checked
    sweep = sg.SurrogateSweep(net, gen, max_abs_err=1.0, check_every=1)
    kinds = [sweep(d, p)[1] for d, p in zip(deltas, pts)]
    assert kinds == ["surrogate"] * 4 and len(sweep.checked) == 4 and sweep.trusted
    # a budget nothing can meet: the first check fails, that point and all later ones are the engine's
    sweep = sg.SurrogateSweep(net, gen, max_abs_err=0.0, check_every=1)
    out = [sweep(d, p) for d, p in zip(deltas, pts)]
    assert [k for _, k in out] == ["engine"] * 4 and not sweep.trusted
    for (xh, _), d, p in zip(out, deltas, pts):
        st = sg.schedule.ionize_setup(gen.n, gen.box_len, p["z"], zeta=p["zeta"], t_vir_min=p["t_vir"],
                                      R_max=p["R_max"], cosmo=gen.cosmo, table=gen.table)
        ref, _ = gen.plan.run(d, st)
        assert torch.equal(xh, ref)
    # trust lost to a bad check comes back once later checks bring the mean error under budget
    sweep = sg.SurrogateSweep(net, gen, max_abs_err=1.0, check_every=2)
    sweep.checked.append(1.2)
    kinds = [sweep(d, p)[1] for d, p in zip(deltas[:3], pts[:3])]
    assert kinds == ["engine", "surrogate", "surrogate"], (kinds, sweep.checked)
    # outside the training ranges the surrogate is never asked
    sweep = sg.SurrogateSweep(net, gen, max_abs_err=1.0, check_every=0)
    far = dict(pts[0], zeta=200.0)
    assert sweep(deltas[0], far)[1] == "engine" and sweep.fallbacks == 1


def test_features_kernel_and_cached_weights(sg):
    # the fused input kernel: channel 0 = bf16(delta * scale) rounded to nearest even, channels
    # 1..4 the parameter constants, the rest zero; the BF16 weight copies follow in-place updates
    cosm = module("cosmology")
    n = 32
    delta = torch.randn((n,) * 3, device="cuda") * 2.0
    z, zeta, rmax, tvir = 8.0, 30.0, 15.0, 2e4
    f = sg.features(delta, z, zeta, rmax, tvir, smoothing=())
    scale = np.float32(1.0 / (4.0 * cosm.growth_factor(z, cosm.BASELINE_COSMO)))
    ref0 = (delta * torch.tensor(float(scale), device="cuda")).to(torch.bfloat16)
    assert torch.equal(f[..., 0], ref0)
    const = torch.tensor([zeta / 80.0, rmax / 50.0, np.log10(tvir) - 4.0, (z - 6.0) / 4.0]).to(torch.bfloat16)
    assert torch.equal(f[..., 1:5], const.cuda().expand(n, n, n, 4))
    assert not f[..., 5:].any()
    # with smoothed channels: channels 5..8 = bf16(delta smoothed with the top hat at 4, 8, 16, 32
    # cells, times the same scale), the first five unchanged, the rest zero
    fs = sg.features(delta, z, zeta, rmax, tvir)
    assert torch.equal(fs[..., :5], f[..., :5]) and not fs[..., 9:].any()
    d64 = delta.double().cpu().numpy()
    X = np.fft.rfftn(d64)
    k = np.sqrt(np.fft.fftfreq(n)[:, None, None] ** 2 + np.fft.fftfreq(n)[None, :, None] ** 2
                + np.fft.rfftfreq(n)[None, None, :] ** 2) * 2 * np.pi       # per cell
    from oracle import es_oracle as O
    for j, R in enumerate(sg.SMOOTH_CELLS):
        ref = np.fft.irfftn(X * O.rtophat(k * R), s=(n, n, n), axes=(0, 1, 2)) * float(scale)
        got = fs[..., 5 + j].float().cpu().numpy()
        assert np.abs(got - ref).max() <= 8e-3 * np.abs(ref).max() + 1e-6, (R, np.abs(got - ref).max())
    net = sg.SurrogateNet(seed=0)
    w0 = net.bf16_weights()
    assert net.bf16_weights() is w0
    net.w[3].mul_(0.5)
    w1 = net.bf16_weights()
    assert w1 is not w0 and torch.equal(w1[3], net.w[3].to(torch.bfloat16))
