"""The warm-start U-Net's CUDA kernels against a PyTorch CPU fp32 reference
of the same network (BF16-rounded convolution weights, as the GPU uses)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ref_forward(torch, params, x, L, c0, leaves, cin=1):
    """Same network on the CPU; the 3x3 weights are rounded to BF16 as the
    GPU uses them and become float leaves (the gradient of a dtype cast would
    itself be rounded).  ``leaves`` receives the leaves in parameter order."""
    F = torch.nn.functional
    off = [0]

    def take(co, ci, k, round_bf16=True):
        n = co * ci * k * k
        w = params[off[0]:off[0] + n].view(co, ci, k, k)
        off[0] += n
        b = params[off[0]:off[0] + co]
        off[0] += co
        if round_bf16:
            w = w.to(torch.bfloat16).float()
        w = w.detach().clone().requires_grad_()
        b = b.detach().clone().requires_grad_()
        leaves.extend([w, b])
        return w, b

    ch = [c0 << l for l in range(L)]
    enc = [(take(ch[l], cin if l == 0 else ch[l - 1], 3), take(ch[l], ch[l], 3)) for l in range(L)]
    dec = {}
    for l in range(L - 2, -1, -1):
        dec[l] = (take(ch[l], ch[l + 1] + ch[l], 3), take(ch[l], ch[l], 3))
    wo, bo = take(1, c0, 1, round_bf16=False)
    es = []
    h = x
    for l in range(L):
        (wa, ba), (wb, bb) = enc[l]
        a = F.relu(F.conv2d(h, wa, ba, padding=1))
        e = F.relu(F.conv2d(a, wb, bb, padding=1))
        es.append(e)
        if l < L - 1:
            h = F.avg_pool2d(e, 2)
    d = es[L - 1]
    for l in range(L - 2, -1, -1):
        u = F.interpolate(d, scale_factor=2, mode="nearest")
        (wc, bc), (wd, bd) = dec[l]
        da = F.relu(F.conv2d(torch.cat([u, es[l]], 1), wc, bc, padding=1))
        d = F.relu(F.conv2d(da, wd, bd, padding=1))
    return F.conv2d(d, wo, bo)


@pytest.fixture
def tensor_cores(request):
    from msot_gb300 import _lib
    _lib.check(_lib.load().msot_tune_set(b"unet_tensor_cores", request.param))
    yield request.param
    _lib.check(_lib.load().msot_tune_set(b"unet_tensor_cores", 1))


# tensor cores: layers with >= 8 input and a multiple of 32 output channels
# (all but the first in the 4-level, 32-channel net); their activations are
# rounded to TF32 (2^-11 relative), hence the looser bars (the gradients
# pass through every level twice: 1e-2).  cin = 2: the two-channel input of
# the trajectory warm start
@pytest.mark.parametrize("tensor_cores", [0, 1], indirect=True)
@pytest.mark.parametrize("L,c0,side,n,cin", [(3, 4, 32, 2, 1), (4, 8, 32, 3, 1), (1, 8, 16, 2, 1),
                                             (4, 32, 64, 2, 1), (2, 32, 40, 1, 1),
                                             (3, 8, 32, 2, 2), (4, 32, 64, 2, 2)])
def test_unet_forward_and_gradients_match_torch_reference(cuda, tensor_cores, L, c0, side, n,
                                                          cin):
    import torch
    from msot_gb300.warmstart import UNet
    tc = tensor_cores and c0 * (1 << (L - 1)) >= 32
    bar_out, bar_grad = (3e-3, 1e-2) if tc else (1e-4, 5e-4)
    net = UNet(levels=L, base_channels=c0, side=side, max_batch=4, seed=7, in_channels=cin)
    rng = np.random.default_rng(1)
    x = rng.standard_normal((n, cin, side, side)).astype(np.float32)
    t = rng.standard_normal((n, 1, side, side)).astype(np.float32)
    p = torch.tensor(net.get_params())
    leaves = []
    out_ref = _ref_forward(torch, p, torch.tensor(x), L, c0, leaves, cin)
    out = net.forward(x).cpu()
    net.check()
    assert float((out - out_ref.detach()).norm() / out_ref.detach().norm()) < bar_out
    loss_ref = ((out_ref - torch.tensor(t)) ** 2).mean()
    loss_ref.backward()
    # _ref_forward takes the blocks in the parameter layout's order
    g_ref = torch.cat([v.grad.reshape(-1) for v in leaves]).numpy()
    loss, g = net.gradients(x, t)
    net.check()
    lr = float(loss_ref.detach())
    assert abs(loss - lr) / lr < bar_out
    assert np.linalg.norm(g - g_ref) / np.linalg.norm(g_ref) < bar_grad


def test_unet_training_reduces_loss(cuda):
    # learn a fixed smoothing of the input: the loss must drop by 10x
    import torch
    from msot_gb300.warmstart import UNet
    net = UNet(levels=3, base_channels=8, side=32, max_batch=8, seed=3)
    rng = np.random.default_rng(2)
    x = torch.tensor(rng.standard_normal((8, 1, 32, 32)).astype(np.float32), device="cuda")
    k = torch.ones(1, 1, 3, 3, device="cuda") / 9.0
    t = torch.nn.functional.conv2d(x, k, padding=1)
    first = net.train_step(x, t, lr=3e-3)
    for _ in range(300):
        last = net.train_step(x, t, lr=3e-3)
    assert last < 0.1 * first


def _ws_model(n, max_batch):
    from msot_gb300 import Discretization, MSOTmodel, Probe
    from msot_gb300.synthetic import gauss_pulse_eir
    h = 0.2e-3 * (n - 1) / 2
    probe = Probe(n_det=256, radius=0.040, angular_coverage=135.0, fs=4e7, n_samples=2030,
                  delay=0.0, eir=gauss_pulse_eir(), eir_length=257)
    return MSOTmodel(probe, Discretization([-h, h], n), 1500.0, False, True, 0, 1e5, 12e6, None,
                     max_batch=max_batch)


def test_learned_warm_start_gain(cuda):
    # trained on pairs of the plain solver (10-iteration iterate -> 200-iteration
    # solution), the network's start must beat the iterate it was given and,
    # 10 iterations on, the plain solve of the same total iteration count,
    # measured against a 1500-iteration solve
    import torch
    from msot_gb300 import rec_nn_with_L2_reg
    from msot_gb300.synthetic import phantom_batch
    from msot_gb300.warmstart import LearnedWarmStart
    lam = 1e-2
    model = _ws_model(64, 64)
    ws = LearnedWarmStart(model, lam, levels=4, base_channels=32, max_batch=16, input_iters=10)
    f, t, b = ws.make_pairs(phantom_batch(model.Discretization, 2048 + 32, seed=1), 200, seed=2)
    ws.fit(f[:2048], t[:2048], 2500, batch=16, lr=2e-3)
    bt = b[2048:]
    xs = rec_nn_with_L2_reg(model, bt, 1500, lam)[0]
    err = lambda x: float((x - xs).norm() / xs.norm())
    w0, _, fell = ws.start(bt)
    assert not bool(fell.any())
    e_in = err(rec_nn_with_L2_reg(model, bt, 10, lam)[0])
    e_pred = err(w0)
    e_warm = err(ws.solve(bt, 10)[0])
    e_plain = err(rec_nn_with_L2_reg(model, bt, 20, lam)[0])
    assert e_pred < 0.75 * e_in, (e_pred, e_in)
    assert e_warm < 0.85 * e_plain, (e_warm, e_plain)


def test_learned_warm_start_falls_back_to_zero_start(cuda):
    # a start worse than zero (objective above |b|^2) is replaced by the zero
    # start: the solve then equals the plain one
    import torch
    from msot_gb300 import rec_nn_with_L2_reg
    from msot_gb300.synthetic import phantom_batch
    from msot_gb300.warmstart import LearnedWarmStart
    model = _ws_model(32, 4)
    ws = LearnedWarmStart(model, 1e-2, levels=3, base_channels=8, max_batch=4)
    x = phantom_batch(model.Discretization, 2, seed=5)
    b = model.forward(x)
    bad = 100.0 * x.max() * torch.rand((2, 32, 32), device="cuda")
    # a regularised solution (the phantom itself can score above the zero
    # start once lambda |x|^2 is counted)
    good = rec_nn_with_L2_reg(model, b, 50, 1e-2)[0]
    w, v, fell = ws.start(b, torch.stack([bad[0], good[1]]))
    assert fell.tolist() == [True, False]
    assert float(w[0].abs().max()) == 0.0 and float(v[0].abs().max()) == 0.0
    rec, fell = ws.solve(b, 5, torch.stack([bad[0], good[1]]))
    plain = rec_nn_with_L2_reg(model, b, 5, 1e-2)[0]
    assert float((rec[0] - plain[0]).norm() / plain[0].norm()) < 1e-5


def test_waveeq_input_lines_up_with_the_image(cuda):
    # the backproject_waveeq input (x mirror of backproject_waveeq.m:49
    # undone) correlates with the phantom; the mirrored image does not
    import torch
    from msot_gb300 import Discretization, MSOTmodel, Probe
    from msot_gb300.synthetic import gauss_pulse_eir
    from msot_gb300.warmstart import LearnedWarmStart
    n = 48
    h = 0.2e-3 * (n - 1) / 2
    probe = Probe(n_det=64, radius=0.02, angular_coverage=135.0, fs=4e7, n_samples=1200,
                  eir=gauss_pulse_eir(), eir_length=257)
    model = MSOTmodel(probe, Discretization([-h, h], n), 1500.0, model_normalization_factor=1.0,
                      max_batch=2)
    img = np.zeros((1, n, n), dtype=np.float32)
    img[0, 10:16, 30:40] = 1.0
    img[0, 30:34, 8:12] = 2.0
    b = model.forward(torch.tensor(img, device="cuda"))
    ws = LearnedWarmStart(model, 1e-2, levels=3, base_channels=8, max_batch=2,
                          backprojection="waveeq")
    f = ws.features(b)[0][0, 0].cpu().numpy()
    corr = lambda a, c: float(np.corrcoef(a.ravel(), c.ravel())[0, 1])
    assert corr(f, img[0]) > 0.3
    assert abs(corr(f[::-1, :], img[0])) < 0.1


def test_l2_state_continuation_equals_the_plain_solve(cuda):
    # msot_rec_nn_with_L2_reg_state: k1 iterations, then k2 more from the
    # returned (image, multiplier), is the k1 + k2 iteration solve
    import torch
    from msot_gb300 import rec_nn_with_L2_reg
    from msot_gb300.synthetic import phantom_batch
    model = _ws_model(32, 4)
    b = model.forward(phantom_batch(model.Discretization, 3, seed=8))
    plain = rec_nn_with_L2_reg(model, b, 7, 1e-2)[0]
    v = torch.empty_like(plain)
    w3 = rec_nn_with_L2_reg(model, b, 3, 1e-2, v_out=v)[0]
    assert float((w3 - rec_nn_with_L2_reg(model, b, 3, 1e-2)[0]).abs().max()) == 0.0
    w7 = rec_nn_with_L2_reg(model, b, 4, 1e-2, x0=w3, v0=v.clone(), v_out=v)[0]
    assert float((w7 - plain).norm() / plain.norm()) < 1e-6


def test_trajectory_features(cuda):
    # input_iters = 4, trajectory = 1: channel 0 is the 4-iteration iterate,
    # channel 1 its last step x_4 - x_3, both over the rms of x_4
    import torch
    from msot_gb300 import rec_nn_with_L2_reg
    from msot_gb300.synthetic import phantom_batch
    from msot_gb300.warmstart import LearnedWarmStart
    model = _ws_model(32, 4)
    b = model.forward(phantom_batch(model.Discretization, 3, seed=9))
    ws = LearnedWarmStart(model, 1e-2, levels=3, base_channels=8, max_batch=4, input_iters=4,
                          trajectory=1)
    f, s = ws.features(b)
    assert tuple(f.shape) == (3, 2, 32, 32)
    x4 = rec_nn_with_L2_reg(model, b, 4, 1e-2)[0]
    x3 = rec_nn_with_L2_reg(model, b, 3, 1e-2)[0]
    sc = s.view(-1, 1, 1)
    assert float((f[:, 0] * sc - x4).norm() / x4.norm()) < 1e-6
    assert float((f[:, 1] * sc - (x4 - x3)).norm() / (x4 - x3).norm()) < 1e-5
    pairs = ws.make_pairs(phantom_batch(model.Discretization, 4, seed=10), 10, seed=11)
    ws.fit(pairs[0], pairs[1], 3, batch=4)
    rec, fell = ws.solve(b, 2)
    assert tuple(rec.shape) == (3, 32, 32) and bool(torch.isfinite(rec).all())
