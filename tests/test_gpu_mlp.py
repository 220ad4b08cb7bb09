"""SNR-screen MLP: GPU forward/backward against the CPU float64 model, training, and the screen's
gain in the forecast pipeline."""
import numpy as np
import pytest

from gwfast_gb300 import _lib, pipeline, synthetic
from gwfast_gb300 import waveforms as W
from gwfast_gb300.screen import SNRScreen
from gwfast_gb300.signal import event_array
from oracle import mlp_oracle as M

pytestmark = pytest.mark.gpu


def params(n, seed):
    return event_array(synthetic.screen_population(n, seed=seed))


@pytest.mark.parametrize('hidden,layers,n', [(32, 2, 300), (256, 4, 600)])
def test_mlp_gradients_match_cpu(gpu_lib, hidden, layers, n):
    """GPU loss and gradients (tensor-core GEMMs for the hidden-to-hidden layers, tcgen05 kind::f16)
    against the float64 model with the same BF16 roundings."""
    rng = np.random.default_rng(hidden)
    mlp = _lib.MLP(hidden=hidden, layers=layers, seed=3)
    p = params(n, 11)
    t = rng.normal(1.0, 1.5, n)
    loss_g, g_gpu = mlp.gradients(p, t)          # sets the standardisation from these events
    w, norm = mlp.get_weights(), mlp.get_norm().astype(np.float64)
    loss_c, g_cpu = M.forward_backward(w, norm, p, t, hidden, layers)
    rel = np.linalg.norm(g_gpu - g_cpu) / np.linalg.norm(g_cpu)
    print('hidden %d layers %d: loss %.6e vs %.6e, gradient relative error %.2e' % (hidden, layers, loss_g, loss_c, rel))
    assert abs(loss_g - loss_c) <= 1e-5 * loss_c
    # the hidden-to-hidden layers take BF16 operands on the tensor cores; where the GPU's FP32 sum and
    # the oracle's float64 sum of a pre-activation straddle a BF16 rounding boundary, that element
    # differs by one BF16 ulp (2^-8 relative): 1.6e-5 (32 wide) and 1.0e-4 (256 wide) measured
    assert rel < 3e-4


@pytest.mark.parametrize('hidden,layers', [(256, 4), (64, 2), (64, 1)])
def test_mlp_predict_matches_cpu(gpu_lib, hidden, layers):
    """Inference (one fused kernel per 128 events: features and input layer on the CUDA cores, the
    hidden-to-hidden layers chained through tensor memory with the activations resident in shared
    memory, the output layer in the last epilogue) against the float64 model with the same BF16
    roundings, on random weights of realistic scale."""
    rng = np.random.default_rng(hidden + layers)
    mlp = _lib.MLP(hidden=hidden, layers=layers, seed=7)
    p = params(3000, 41)
    mlp.gradients(p, rng.normal(1.0, 1.5, p.shape[1]))   # sets the standardisation
    w = mlp.get_weights()
    w = w + rng.normal(0.0, 0.05, w.shape).astype(np.float32)   # non-zero biases as well
    mlp.set_weights(w)
    y = mlp.predict(p)
    yc = M.predict(mlp.get_weights(), mlp.get_norm().astype(np.float64), p, hidden, layers)
    d = np.abs(y - yc)
    sc = max(1.0, np.std(yc))
    print('hidden %d layers %d: predict vs float64 model max %.2e p99 %.2e median %.2e (scale %.2f)'
          % (hidden, layers, d.max(), np.percentile(d, 99), np.median(d), np.std(yc)))
    # typical events differ by the FP32 sums alone (~1e-7); a few differ more where a hidden activation
    # lies on a BF16 rounding boundary and the GPU and the model round it to neighbouring BF16 values
    # (one BF16 ulp, 2^-8 relative), which the following layers carry to the output (measured max:
    # 5.5e-3 with three BF16 layers, 3.6e-4 with one, 1.3e-6 with none)
    assert np.median(d) < 1e-5 * sc
    assert np.percentile(d, 99) < 1e-3 * sc
    assert d.max() < 2e-2 * sc


def test_mlp_training_reduces_loss_and_predicts(gpu_lib):
    p = params(20000, 21)
    f = M.features(p)
    t = 0.8 * f[:, 0] - f[:, 2] + 0.5 * f[:, 6] ** 2 + 0.3 * f[:, 5]      # a smooth target of the features
    mlp = _lib.MLP(hidden=64, layers=2, seed=5)
    l0, _ = mlp.gradients(p, t)
    loss = mlp.train(p, t, epochs=20, batch=2048, lr=3e-3)
    pred = mlp.predict(p)
    rms = np.sqrt(np.mean((pred - t) ** 2))
    print('initial loss %.3e, final %.3e, rms %.3e' % (l0, loss, rms))
    assert loss < 1e-2 * l0
    assert abs(rms ** 2 - loss) < 0.5 * loss + 1e-6
    # predictions agree with the CPU model with the trained weights
    _, _ = M.forward_backward(mlp.get_weights(), mlp.get_norm().astype(np.float64), p[:, :100], t[:100], 64, 2)


def test_screen_gain_and_audit(gpu_lib):
    net = synthetic.make_network(W.IMRPhenomD(), earth=True)
    train = synthetic.screen_population(40000, seed=31)
    screen = SNRScreen(net, hidden=256, layers=4, seed=1)
    loss = screen.fit(dict(train), res=1000, epochs=40, batch=4096, lr=2e-3)
    ev = synthetic.screen_population(20000, seed=32)
    exact_snr = net.SNR(dict(ev), res=1000, precision='fp32')
    pred = screen.predict_ln_snr(dict(ev))
    err = pred - np.log(exact_snr)
    near = np.abs(np.log(exact_snr) - np.log(12.)) < 1.0
    r0 = pipeline.compute_errs(net, dict(ev), snr_th=12., res=1000, precision='mixed', sky_area=False)
    r1 = pipeline.compute_errs(net, dict(ev), snr_th=12., res=1000, precision='mixed', sky_area=False, screen=screen)
    info = r1['screen']
    print('train loss %.3e; held-out ln SNR error rms %.3f (%.3f near threshold), max |err| %.3f; screen %s; '
          'detected %d (exact path %d)' % (loss, np.sqrt(np.mean(err ** 2)), np.sqrt(np.mean(err[near] ** 2)),
                                            np.abs(err).max(), info, r1['detected'].sum(), r0['detected'].sum()))
    assert info['audit_missed_detections'] == 0
    assert info['exact_snr_fraction'] < 0.5          # the gain: most events need no exact SNR
    # recall against the exact path (a detection is lost only if its prediction is off by more than
    # the band and it is not in the audit sample), and few false detections
    recall = np.mean(r1['detected'][r0['detected']])
    precision = np.mean(exact_snr[r1['detected']] > 12.)
    print('recall %.4f precision %.4f' % (recall, precision))
    assert recall >= 0.99 and precision >= 0.95
