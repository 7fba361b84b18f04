"""Learned initial guess: the library's BF16 tensor-core forward and backward
kernels against the float64 CPU oracle of the same network (oracle/net_oracle.py,
which rounds to BF16 where the GPU stores BF16), training, and the solver hook.

Tolerances: the network output within 1e-2 relative L2 of the oracle, the
loss within 2e-3, every layer's weight and bias gradient within 3e-2 relative
L2 (BF16 operands; the remaining differences are FP32 accumulation order and
the BF16 roundings it occasionally flips)."""
import numpy as np
import pytest

from oracle import net_oracle as no

pytestmark = pytest.mark.gpu


def _dev(a, dtype=None):
    import torch
    t = torch.from_numpy(np.ascontiguousarray(np.asarray(a).ravel(order="F")))
    return (t.to(dtype) if dtype is not None else t).cuda()


def _tiny(rng, nx=16, ny=16, nz=8):
    x, y, z = np.meshgrid(np.linspace(-1, 1, nx), np.linspace(-1, 1, ny), np.linspace(-1, 1, nz), indexing="ij")
    fluid = (((x / 0.5) ** 2 + (y / 0.4) ** 2 + (z / 0.6) ** 2) > 1).astype(np.uint8)
    mx, my, mz = (rng.uniform(0.3, 1.0, n).astype(np.float32) for n in (nx, ny, nz))
    rhs = (rng.standard_normal((nx, ny, nz)) * (rng.random((nx, ny, nz)) < 0.3)).astype(np.float32)
    target = (np.sin(2 * x) * np.cos(y) + 0.3 * z + 0.05 * rng.standard_normal((nx, ny, nz))).astype(np.float32)
    return fluid, mx, my, mz, rhs, target


def _layers():
    o = 0
    for ci, _, co, _, _ in no.SPEC:
        nw = 27 * co * ci
        yield slice(o, o + nw), slice(o + nw, o + nw + co)
        o += nw + co


@pytest.mark.parametrize("shape", [(16, 16, 8), (128, 8, 8), (256, 8, 8)])
def test_forward_and_gradients_match_oracle(gpu_lib, shape):
    """Layers whose rows are multiples of 128 voxels run on the tcgen05
    tensor-core kernel (TMEM accumulators), the others on the mma.sync kernel:
    (128, 8, 8) the full-resolution layers (16 and 48 output channels),
    (256, 8, 8) also the half-resolution ones (32 and 80); (16, 16, 8) none."""
    from flowfpmpp_gb300.learned import LearnedGuess
    rng = np.random.default_rng(5)
    net = LearnedGuess(seed=11)
    p = net.params()
    assert p.size == no.param_count()
    for _, sb in _layers():
        p[sb] = rng.normal(0, 0.05, sb.stop - sb.start)
    last_w, last_b = list(_layers())[-1]
    p[last_b.start + 1:last_b.stop] = 0.0  # the head keeps output channel 0 only
    net.set_params(p)
    fluid, mx, my, mz, rhs, target = _tiny(rng, *shape)
    nx, ny, nz = fluid.shape
    args = (nx, ny, nz, _dev(fluid), _dev(mx), _dev(my), _dev(mz), _dev(rhs))
    y = net.forward(*args).cpu().numpy().reshape((nx, ny, nz), order="F")
    loss = net.backward(*args, _dev(target))
    g = net.grads()
    y_o, loss_o, g_o = no.output_and_grads(p, fluid, mx, my, mz, rhs, target)
    assert np.linalg.norm(y - y_o) <= 1e-2 * np.linalg.norm(y_o)
    assert abs(loss - loss_o) <= 2e-3, (loss, loss_o)
    for n, (sw, sb) in enumerate(_layers()):
        # relative to the layer's whole gradient where a part is ~0 in exact
        # arithmetic (the head bias: the loss is offset free)
        scale = np.linalg.norm(g_o[sw.start:sb.stop])
        for sl, what in ((sw, "weights"), (sb, "bias")):
            ref = g_o[sl]
            err = np.linalg.norm(g[sl] - ref) / max(np.linalg.norm(ref), 1e-2 * scale)
            assert err <= 3e-2, (n, what, err)


def test_training_lowers_the_loss(gpu_lib):
    from flowfpmpp_gb300.learned import LearnedGuess
    rng = np.random.default_rng(6)
    net = LearnedGuess(seed=2)
    fluid, mx, my, mz, rhs, target = _tiny(rng)
    nx, ny, nz = fluid.shape
    args = (nx, ny, nz, _dev(fluid), _dev(mx), _dev(my), _dev(mz), _dev(rhs), _dev(target))
    first = net.train_step(*args, 3e-3)
    for _ in range(60):
        last = net.train_step(*args, 3e-3)
    assert last < 0.5 * first, (first, last)


def _problem(nx, ny, nz, seed, axis=0):
    from flowfpmpp_gb300 import learned as lg
    rng = np.random.default_rng(seed)
    ax, ay, az = lg.training_grid(nx, ny, nz)
    return lg.DeviceProblem(lg.frame_for(lg.random_bodies(rng, ax, ay, az), ax, ay, az, axis))


def test_learned_solve_matches_plain_solve(gpu_lib):
    """With any network (here an untrained one) the learned solve reaches the
    tolerance and the same potential as the plain solve (1e-9 relative)."""
    from flowfpmpp_gb300.learned import LearnedGuess
    net = LearnedGuess(seed=4)
    p = _problem(32, 32, 16, seed=8, axis=1)
    for method in ("pcg", "pcg_mixed"):
        ref, sw0, r0, _ = p.solve(method, tol=1e-10)
        phi, sw1, r1, fb = p.solve(method, tol=1e-10, net=net)
        assert r0 <= 1e-10 and r1 <= 1e-10, (method, r0, r1)
        ref, phi = ref.cpu().numpy(), phi.cpu().numpy()
        assert np.abs(phi - ref).max() <= 1e-9 * np.abs(ref).max(), method
        assert fb in (0, 1)


def test_learned_flexible_cg(gpu_lib):
    """The flexible CG with the network as preconditioner reaches the
    tolerance and the plain FP64 PCG potential (1e-9 relative), with an
    untrained network as well (the diagonal step keeps the preconditioner
    useful; a stalled run is finished by FP64 PCG); without the network the
    method is refused."""
    from flowfpmpp_gb300 import FpmError
    from flowfpmpp_gb300.learned import LearnedGuess
    p = _problem(32, 32, 16, seed=8, axis=1)
    ref, sw0, r0, _ = p.solve("pcg", tol=1e-10)
    ref = ref.cpu().numpy()
    for net in (LearnedGuess(seed=4), LearnedGuess(seed=9)):
        phi, sw1, r1, _ = p.solve("fcg_learned", tol=1e-10, net=net)
        print(f"fcg_learned: {sw1} iterations (plain PCG {sw0}), residual {r1:.2e}")
        assert r1 <= 1e-10
        assert np.abs(phi.cpu().numpy() - ref).max() <= 1e-9 * np.abs(ref).max()
    with pytest.raises(FpmError):
        p.solve("fcg_learned", tol=1e-10)


def test_trained_network_guess(gpu_lib):
    """What the committed trained network gains, on unseen bodies at the
    training size: its output is within 50 % (relative L2 over fluid cells,
    means removed, best scale) of the converged potential, the learned solve
    converges without a fallback, and its PCG iteration count stays within
    10 % of the solve from phi = 0 (a guess of this accuracy is worth about
    half a decade of a ten-decade solve, while its error is concentrated
    near the body surface, where PCG converges last; the measured counts are
    printed)."""
    import os
    from flowfpmpp_gb300 import learned as lg
    if not os.path.exists(lg.WEIGHTS):
        pytest.skip("no trained weights committed")
    net = lg.LearnedGuess.load()
    for seed in (1001, 1002, 1003):
        p = _problem(128, 128, 64, seed=seed, axis=seed % 3)
        fluid, mx, my, mz, b = p.inputs()
        y = net.forward(p.nx, p.ny, p.nz, fluid, mx, my, mz, b).double().cpu().numpy()
        ref, sw0, r0, _ = p.solve("pcg", tol=1e-10)
        phi = p.interior(ref).cpu().numpy()
        f = fluid.cpu().numpy() != 0
        yc, tc = y[f] - y[f].mean(), phi[f] - phi[f].mean()
        rel = np.linalg.norm(tc - (yc @ tc) / (yc @ yc) * yc) / np.linalg.norm(tc)
        _, sw1, r1, fb = p.solve("pcg", tol=1e-10, net=net)
        msg = f"body {seed}: guess error {rel:.3f}, PCG iterations {sw0} -> {sw1}"
        if seed == 1001:  # the flexible CG with the network, once (it is slow)
            _, sw2, r2, _ = p.solve("fcg_learned", tol=1e-10, net=net)
            msg += f", flexible CG with the network {sw2}"
            assert r2 <= 1e-10
        print(msg)
        assert rel < 0.5, rel
        assert r1 <= 1e-10 and fb == 0
        assert sw1 <= 1.1 * sw0, (sw0, sw1)
