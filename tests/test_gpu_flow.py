"""The learned proposal: CUDA training kernels against the CPU restatement,
and what the trained flow gains over the plain ellipsoidal sampler."""
import math

import numpy as np
import pytest

import lensed_gb300 as lg
from oracle import flow_oracle

pytestmark = pytest.mark.gpu


def _grad_case(bf16):
    import ctypes as C

    d, layers, width, hidden, n = 5, 4, 16, 2, 64
    rng = np.random.Generator(np.random.PCG64(1))
    npar = lg.lib().lg_flow_nparams(d, layers, width, hidden)
    params = (rng.normal(size=npar) * 0.3).astype(np.float32)
    x = rng.normal(size=(n, d)).astype(np.float32)
    loss = C.c_float()
    grad = np.zeros(npar, np.float32)
    rc = lg.lib().lg_flow_loss_grad(0, d, layers, width, hidden, bf16, params.ctypes.data_as(C.POINTER(C.c_float)),
                                    x.ctypes.data_as(C.POINTER(C.c_float)), n, C.byref(loss),
                                    grad.ctypes.data_as(C.POINTER(C.c_float)))
    assert rc == 0
    want_loss, want_grad = flow_oracle.loss_grad(params.astype(np.float64), x.astype(np.float64), d, layers, width,
                                                 hidden)
    err = np.abs(grad - want_grad).max() / np.abs(want_grad).max()
    return loss.value, want_loss, err


def test_flow_gradients_fp32_activations(native):
    l, wl, err = _grad_case(0)
    assert abs(l - wl) <= 1e-4 * abs(wl)
    assert err <= 1e-4, err


def test_flow_gradients_bf16_activations(native):
    l, wl, err = _grad_case(1)
    assert abs(l - wl) <= 2e-2 * abs(wl)
    assert err <= 5e-2, err


def _tc_case(n, seed=1, d=13, layers=4):
    import ctypes as C

    width, hidden = 128, 2
    rng = np.random.Generator(np.random.PCG64(seed))
    npar = lg.lib().lg_flow_nparams(d, layers, width, hidden)
    params = (rng.normal(size=npar) * 0.05).astype(np.float32)
    x = rng.normal(size=(n, d)).astype(np.float32)
    loss = C.c_float()
    grad = np.zeros(npar, np.float32)
    rc = lg.lib().lg_flow_loss_grad(0, d, layers, width, hidden, 2, params.ctypes.data_as(C.POINTER(C.c_float)),
                                    x.ctypes.data_as(C.POINTER(C.c_float)), n, C.byref(loss),
                                    grad.ctypes.data_as(C.POINTER(C.c_float)))
    assert rc == 0, lg.lib().lg_last_error(None)
    return params, x, loss.value, grad


@pytest.mark.parametrize("n", [128, 200, 256])
def test_flow_gradients_tensor_core_training_step(native, n):
    """lg_flow_step_tc (tcgen05: BF16 operands, FP32 accumulators in tensor
    memory, transposed operands for the backward products) against the CPU
    restatement with the same rounding points; one, two ragged and two full
    128-row blocks.  Against the FP32 restatement the BF16 rounding moves
    the gradient by under 1%."""
    d, layers, width, hidden = 13, 4, 128, 2
    params, x, l, g = _tc_case(n)
    wl, wg = flow_oracle.loss_grad_tc(params.astype(np.float64), x.astype(np.float64), d, layers, width, hidden)
    err = np.abs(g - wg).max() / np.abs(wg).max()
    print(f"n {n}: loss {l:.6f} vs {wl:.6f}; max grad error {err:.2e} of the largest component")
    assert abs(l - wl) <= 1e-4 * abs(wl)
    assert err <= 2e-3, err
    fl, fg = flow_oracle.loss_grad(params.astype(np.float64), x.astype(np.float64), d, layers, width, hidden)
    assert np.abs(g - fg).max() / np.abs(fg).max() <= 2e-2
    # deterministic: the same bits again
    _, _, l2, g2 = _tc_case(n)
    assert l2 == l and np.array_equal(g2, g)


def test_tensor_core_training_matches_fp32_training(native):
    """A retraining with tensor-core steps lowers the held-out loss about as
    far as one with the FP32-weight steps (same points, epochs and early
    stopping)."""
    rng = np.random.Generator(np.random.PCG64(4))
    base = rng.normal(size=(1000, 8))
    pts = np.column_stack([base[:, :4], base[:, 4:] * 0.2 + 0.5 * base[:, :4] ** 2])
    flow = dict(layers=8, width=128, hidden=2, epochs=60)
    h_tc, e_tc = lg.flow_fit(pts, train_tc=1, **flow)
    h_32, e_32 = lg.flow_fit(pts, train_tc=0, **flow)
    best_tc, best_32 = np.nanmin(h_tc), np.nanmin(h_32)
    print(f"held-out loss: start {h_tc[0]:.4f}; best tensor-core {best_tc:.4f} ({np.sum(np.isfinite(h_tc)) - 1} "
          f"epochs, kept {e_tc:.3f}); best FP32 {best_32:.4f} ({np.sum(np.isfinite(h_32)) - 1} epochs, kept {e_32:.3f})")
    assert best_tc < h_tc[0] - 0.2 and best_32 < h_32[0] - 0.2
    assert abs(best_tc - best_32) < 0.15 * abs(h_tc[0] - best_32)


def test_tensor_core_training_timeout_is_reported_and_survived(native):
    """wait_tries < 0 with the tensor-core training step (width 128, two
    hidden layers): its first bounded wait gives up, the kernel flags the
    error and stops the retraining, and the fit reports LG_ERR_TIMEOUT; the
    next fit with the default budget trains normally."""
    rng = np.random.Generator(np.random.PCG64(5))
    pts = rng.normal(size=(600, 6))
    flow = dict(layers=4, width=128, hidden=2, epochs=5, train_tc=1)
    with pytest.raises(lg.LensedError) as e:
        lg.flow_fit(pts, wait_tries=-1, **flow)
    assert e.value.code == -5  # LG_ERR_TIMEOUT
    assert "training step" in str(e.value)
    hist, eff = lg.flow_fit(pts, **flow)
    assert np.all(np.isfinite(hist[:2])) and eff > 0


def test_learned_sampler_with_tensor_core_training(native):
    """The sampler with the learned proposal trained by the tensor-core
    steps reaches the closed-form evidence of the curved posterior."""
    d = 4
    exact = 2 * math.log(2 * math.pi * 0.15 * 0.01)
    r = lg.nested_sample_flow(banana, d, nlive=400, batch=512, seed=7, tol=0.1, flow_every=400,
                              flow=dict(layers=8, width=128, hidden=2, train_tc=1))
    print(f"tensor-core training: lnZ {r['logz']:.3f} +- {r['logz_err']:.3f} (exact {exact:.3f}), "
          f"{r['ncall']} calls, {r['n_flow_proposals']} from the flow")
    assert r["n_flow_proposals"] > 0
    assert abs(r["logz"] - exact) < 4 * r["logz_err"] + 0.1


def banana(x):
    """Three curved ridges: x_{2i+1} ~ 0.3 + 1.5 (x_{2i} - 0.5)^2 +- 0.01."""
    ll = np.zeros(x.shape[0])
    for i in range(0, x.shape[1], 2):
        u = (x[:, i] - 0.5) / 0.15
        v = (x[:, i + 1] - 0.3 - 1.5 * (x[:, i] - 0.5) ** 2) / 0.01
        ll += -0.5 * (u * u + v * v)
    return ll


def test_learned_proposal_on_a_curved_posterior(native):
    d = 6
    exact = 3 * math.log(2 * math.pi * 0.15 * 0.01)
    common = dict(nlive=500, batch=512, seed=5, tol=0.1)
    plain = lg.nested_sample(banana, d, **common)
    flow = lg.nested_sample_flow(banana, d, flow_every=500, flow=dict(layers=4, width=64, epochs=60), **common)
    print(f"banana d={d}: exact lnZ {exact:.3f}; ellipsoid {plain['logz']:.3f}+-{plain['logz_err']:.3f} "
          f"calls {plain['ncall']} ({plain['wall_s']:.1f}s); flow {flow['logz']:.3f}+-{flow['logz_err']:.3f} "
          f"calls {flow['ncall']} ({flow['wall_s']:.1f}s), flow proposals {flow['n_flow_proposals']}")
    # the learned bound is used where it is tighter than the ellipsoid, and
    # the evidence stays unbiased (calibrated rejection step)
    assert flow["n_flow_proposals"] > 0
    assert flow["ncall"] < plain["ncall"]
    for r in (plain, flow):
        assert abs(r["logz"] - exact) < 4 * r["logz_err"] + 0.1


def test_learned_sampler_repeats(native):
    """Retraining, proposal refills and latent-radius updates run on their
    own streams; the sampler takes their results at fixed replacement
    counts, so two runs with one seed give the same draws and the same
    evidence bit for bit."""
    common = dict(nlive=300, batch=512, seed=9, tol=0.1, flow_every=300,
                  flow=dict(layers=4, width=64, epochs=40))
    a = lg.nested_sample_flow(banana, 4, **common)
    b = lg.nested_sample_flow(banana, 4, **common)
    assert a["n_flow_proposals"] > 0
    for k in ("logz", "ncall", "niter", "n_flow_proposals", "n_ellipsoid_proposals"):
        assert a[k] == b[k], (k, a[k], b[k])
    assert np.array_equal(a["samples"], b["samples"])


def test_learned_sampler_on_a_lens_model(native):
    """The learned sampler through a GPU context (cube -> priors -> logL on
    the GPU, ellipsoid draws on the GPU): 128^2 SIE + Sersic + sky, 13 free
    parameters.  Its evidence agrees with the plain sampler's within their
    errors and it needs fewer exact likelihood calls."""
    from lensed_gb300 import workloads

    s = workloads.small()
    ctx = lg.Context(s.image, s.weight, s.objects, rule=s.rule, max_batch=1024)
    common = dict(nlive=300, batch=1024, tol=0.1, seed=3)
    plain = ctx.nested(**common)
    flow = ctx.nested(proposal=lg.PROPOSAL_FLOW, flow_every=300, **common)
    ctx.close()
    print(f"lens model: plain {plain['logz']:.3f}+-{plain['logz_err']:.3f} calls {plain['ncall']} "
          f"({plain['wall_s']:.2f}s); flow {flow['logz']:.3f}+-{flow['logz_err']:.3f} calls {flow['ncall']} "
          f"({flow['wall_s']:.2f}s), flow proposals {flow['n_flow_proposals']}")
    assert flow["n_flow_proposals"] > 0
    assert flow["ncall"] < plain["ncall"]
    assert abs(flow["logz"] - plain["logz"]) < 3 * math.hypot(flow["logz_err"], plain["logz_err"])


def test_retraining_lowers_the_held_out_loss(native):
    """One retraining as the sampler runs it (device-side epochs and early
    stopping): on curved, correlated points the held-out negative
    log-likelihood falls well below the identity flow's, and the best epoch
    is the one kept (history[0] is the loss before training)."""
    d = 13
    rng = np.random.Generator(np.random.PCG64(3))
    A = rng.normal(size=(d, d)) * 0.5 + np.eye(d)
    y = rng.uniform(-1, 1, size=(1000, d)) @ A.T
    y[:, 1] += 2 * y[:, 0] ** 2
    hist, eff = lg.flow_fit(y, epochs=40, patience=10)
    print(f"held-out loss before {hist[0]:.3f}, best {np.nanmin(hist):.3f} after {len(hist) - 1} epochs, "
          f"kept fraction {eff:.4f}")
    assert np.nanmin(hist[1:]) < hist[0] - 1.0
    assert len(hist) - 1 <= 40


def _inverse_case(tc, bf16, d=13, layers=8, width=128, hidden=2, M=1000):
    import ctypes as C

    rng = np.random.Generator(np.random.PCG64(7))
    npar = lg.lib().lg_flow_nparams(d, layers, width, hidden)
    params = (rng.normal(size=npar) * 0.08).astype(np.float32)
    z = rng.normal(size=(M, d)).astype(np.float32)
    u = np.zeros((M, d), np.float32)
    ld = np.zeros(M, np.float32)
    P = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
    rc = lg.lib().lg_flow_inverse_check(0, d, layers, width, hidden, bf16, tc, P(params), P(z), M, P(u), P(ld))
    assert rc == 0, lg.lib().lg_last_error(None)
    mode = "tc" if tc else ("bf16" if bf16 else "fp32")
    want_u, want_ld = flow_oracle.inverse(params.astype(np.float64), z.astype(np.float64), d, layers, width,
                                          hidden, mode)
    du = np.abs(u - want_u) / (1 + np.abs(want_u))
    dl = np.abs(ld - want_ld) / (1 + np.abs(want_ld))
    print(f"inverse {mode}: u error max {du.max():.3g} median {np.median(du):.3g}; "
          f"logdet error max {dl.max():.3g} median {np.median(dl):.3g}")
    return du, dl


def test_inverse_fp32_kernel(native):
    du, dl = _inverse_case(tc=0, bf16=0)
    assert du.max() <= 1e-4 and dl.max() <= 1e-4


def test_inverse_tensor_core_kernel(native):
    """The proposals' inverse on tcgen05 (BF16 operands in shared memory,
    FP32 accumulators in tensor memory) against the same map in float64 with
    the same BF16 rounding points: agreement to FP32 accumulation order,
    except where an FP32 difference flips a BF16 rounding downstream."""
    du, dl = _inverse_case(tc=1, bf16=1)
    assert np.median(du) <= 1e-5 and np.median(dl) <= 1e-5
    assert du.max() <= 2e-2 and dl.max() <= 2e-2


def test_learned_proposal_with_a_wrapped_dimension(native):
    """The flow's proposals wrap periodic dimensions into the cube as the
    ellipsoid's do (Gaussian centred on the boundary 0 = 1 of dimension 0)."""
    sigma = 0.05

    def f(x):
        d0 = x[:, 0] - np.round(x[:, 0])
        return -0.5 * (d0 / sigma) ** 2 - 0.5 * np.sum(((x[:, 1:] - 0.5) / sigma) ** 2, axis=1)

    exact = 2.0 * math.log(2 * math.pi * sigma ** 2)
    r = lg.nested_sample_flow(f, 4, nlive=400, batch=512, seed=3, tol=0.1, flow_every=400, wrap=[1, 0, 0, 0],
                              flow=dict(layers=4, width=64, epochs=60, lag=200))
    print(f"wrapped Gaussian d=4: exact {exact:.3f}, flow {r['logz']:.3f}+-{r['logz_err']:.3f}, "
          f"calls {r['ncall']}, flow proposals {r['n_flow_proposals']}")
    assert abs(r["logz"] - exact) < 4 * r["logz_err"] + 0.1


def _draw(ells, B, wrap=None, seed=1):
    """GPU draws in a union of spheres/ellipsoids given as (mu, cov, scale)."""
    import ctypes as C

    d = len(ells[0][0])
    packed, logv = [], []
    for mu, cov, scale in ells:
        L = np.linalg.cholesky(np.asarray(cov, np.float64))
        packed += list(mu) + list(L.ravel()) + [scale]
        logv.append(0.5 * d * math.log(math.pi) - math.lgamma(0.5 * d + 1) + 0.5 * d * math.log(scale)
                    + np.log(np.diag(L)).sum())
    packed = np.array(packed, np.float64)
    logv = np.array(logv, np.float64)
    w = None if wrap is None else np.array(wrap, np.int32)
    out = np.zeros((B, d))
    n = lg.lib().lg_ellipsoid_draw_check(0, d, len(ells), packed.ctypes.data_as(C.POINTER(C.c_double)),
                                         logv.ctypes.data_as(C.POINTER(C.c_double)),
                                         None if w is None else w.ctypes.data_as(C.POINTER(C.c_int)),
                                         out.ctypes.data_as(C.POINTER(C.c_double)), B, seed)
    assert n == B, n
    return out


def test_gpu_ellipsoid_draws_are_uniform(native):
    """The sampler's GPU proposals: uniform in one ball (radial CDF r^d,
    centred), uniform in the union of two overlapping balls (the overlap
    holds its volume share, not twice it), periodic wrapping."""
    d, B = 3, 200000
    x = _draw([([0.5] * d, np.eye(d) * 0.09, 1.0)], B)  # radius 0.3
    r = np.linalg.norm(x - 0.5, axis=1) / 0.3
    assert r.max() <= 1 + 1e-9
    assert np.abs(np.mean(r ** d) - 0.5) < 0.005 and np.abs(x.mean(0) - 0.5).max() < 0.003
    # two balls of radius 0.2, centres 0.2 apart along x: overlap volume share
    c1, c2 = np.array([0.4, 0.5, 0.5]), np.array([0.6, 0.5, 0.5])
    x = _draw([(c1, np.eye(d) * 0.04, 1.0), (c2, np.eye(d) * 0.04, 1.0)], B, seed=3)
    in1 = np.linalg.norm(x - c1, axis=1) <= 0.2 + 1e-12
    in2 = np.linalg.norm(x - c2, axis=1) <= 0.2 + 1e-12
    assert np.all(in1 | in2)
    R, dd = 0.2, 0.2
    lens = math.pi * (4 * R + dd) * (2 * R - dd) ** 2 / 12  # lens-shaped overlap of two balls
    ball = 4 / 3 * math.pi * R ** 3
    share = lens / (2 * ball - lens)
    assert abs(np.mean(in1 & in2) - share) < 0.006, (np.mean(in1 & in2), share)
    # a ball of radius 0.1 across the boundary x0 = 0 of a periodic
    # dimension: the cap below 0 (height 0.05, 5/32 of the ball) re-enters
    # near x0 = 1
    x = _draw([([0.05, 0.5, 0.5], np.eye(d) * 0.01, 1.0)], 100000, wrap=[1, 0, 0], seed=5)
    assert np.all((x >= 0) & (x <= 1))
    assert abs(np.mean(x[:, 0] > 0.5) - 5 / 32) < 0.006, np.mean(x[:, 0] > 0.5)


def test_tensor_core_inverse_timeout_is_reported_and_survived(native):
    """wait_tries < 0: every bounded mbarrier wait of the tensor-core inverse
    gives up at once.  The kernel flags the error and returns (after its own
    copies and MMA work in flight complete and its tensor memory is freed),
    with no hang: a retraining reports LG_ERR_TIMEOUT, the same flow then
    trains normally with the default budget, and a sampler whose flows all
    time out drops them and finishes on the ellipsoid with the right
    evidence."""
    rng = np.random.Generator(np.random.PCG64(3))
    pts = rng.normal(size=(600, 6))
    flow = dict(layers=4, width=64, epochs=5)
    with pytest.raises(lg.LensedError) as e:
        lg.flow_fit(pts, wait_tries=-1, **flow)
    assert e.value.code == -5  # LG_ERR_TIMEOUT
    hist, eff = lg.flow_fit(pts, **flow)  # the device and the library stay usable
    assert np.all(np.isfinite(hist)) and eff > 0
    d = 4
    exact = 2 * math.log(2 * math.pi * 0.15 * 0.01)
    common = dict(nlive=300, batch=512, seed=9, tol=0.1)
    r = lg.nested_sample_flow(banana, d, flow_every=300, flow=dict(wait_tries=-1, **flow), **common)
    plain = lg.nested_sample(banana, d, **common)
    print(f"timeouts: flow proposals {r['n_flow_proposals']}, lnZ {r['logz']:.3f}+-{r['logz_err']:.3f} "
          f"(plain {plain['logz']:.3f}, exact {exact:.3f})")
    assert r["n_flow_proposals"] == 0
    assert abs(r["logz"] - exact) < 4 * r["logz_err"] + 0.1


def test_sampler_configuration_with_learned_proposal(native):
    """The sampler configuration as specified: the 128^2 SIE + Sersic + sky
    model (13 free parameters), nlive = 1000, batches of 1024, the learned
    proposal (8 coupling layers, MLP width 128, 2 hidden layers) retrained
    every 1000 replacements, against the plain ellipsoidal sampler on the
    same GPU, two seeds each: the mean ln Z agree within 0.1 plus three
    standard errors, and the learned sampler needs fewer exact likelihood
    calls."""
    from lensed_gb300 import workloads

    s = workloads.small()
    ctx = lg.Context(s.image, s.weight, s.objects, rule=s.rule, max_batch=1024)
    common = dict(nlive=1000, batch=1024, tol=0.1)
    flow = dict(layers=8, width=128, hidden=2)
    plain = [ctx.nested(seed=sd, **common) for sd in (11, 18)]
    learned = [ctx.nested(seed=sd, proposal=lg.PROPOSAL_FLOW, flow_every=1000, flow=flow, **common) for sd in (11, 18)]
    ctx.close()
    zp = np.mean([r["logz"] for r in plain])
    zl = np.mean([r["logz"] for r in learned])
    se = math.hypot(np.mean([r["logz_err"] for r in plain]), np.mean([r["logz_err"] for r in learned])) / math.sqrt(2)
    cp = np.mean([r["ncall"] for r in plain])
    cl = np.mean([r["ncall"] for r in learned])
    print(f"sampler configuration: plain lnZ {zp:.3f} calls {cp:.0f} wall "
          f"{np.mean([r['wall_s'] for r in plain]):.2f}s; learned lnZ {zl:.3f} calls {cl:.0f} wall "
          f"{np.mean([r['wall_s'] for r in learned]):.2f}s, flow proposals "
          f"{[r['n_flow_proposals'] for r in learned]}; difference {zl - zp:.3f} +- {se:.3f}")
    assert all(r["n_flow_proposals"] > 0 for r in learned)
    assert abs(zl - zp) < 0.1 + 3 * se
    assert cl < cp
