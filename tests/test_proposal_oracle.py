"""The proposal network's FP64 oracle against finite differences, and its
rotation helpers against their definitions (CPU)."""
import numpy as np

from oracle import proposal as PO


def random_quats(rng, n):
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    return np.where(q[:, :1] < 0, -q, q)


def test_oracle_gradients_match_finite_differences():
    rng = np.random.default_rng(4)
    _, total = PO.layout()
    params = rng.normal(scale=0.08, size=total)
    X = rng.random((3, 4096)) * 2.0
    quats = random_quats(rng, 3)
    L, g = PO.loss_and_grads(params, X, quats)
    lay, _ = PO.layout()
    # a few entries of every parameter block
    idx = np.concatenate([o + rng.choice(int(np.prod(s)), 4, replace=False) for o, s in lay])
    eps = 1e-6
    for k in idx:
        p1, p2 = params.copy(), params.copy()
        p1[k] += eps
        p2[k] -= eps
        fd = (PO.loss_and_grads(p1, X, quats)[0] - PO.loss_and_grads(p2, X, quats)[0]) / (2 * eps)
        assert abs(fd - g[k]) <= 1e-5 * max(1.0, abs(g[k])), (k, fd, g[k])


def test_six_d_round_trip_and_friedel_mate():
    rng = np.random.default_rng(1)
    q = random_quats(rng, 50)
    back = PO.six_d_to_quat(PO.quat_to_6d(q))
    np.testing.assert_allclose(np.abs((back * q).sum(1)), 1.0, atol=1e-12)
    # the mate's 6D form is the negative
    np.testing.assert_allclose(PO.quat_to_6d(PO.friedel_mate(q)), -PO.quat_to_6d(q), atol=1e-12)
    # the loss does not tell a rotation from its mate
    o = PO.quat_to_6d(q)
    assert PO.loss(o, -o)[0] == 0.0


def test_inputs_binning():
    rng = np.random.default_rng(2)
    side = 128
    images = rng.poisson(0.5, size=(2, side * side)).astype(np.float32)
    images[0, 5] = -1.0
    mask = (rng.random(side * side) > 0.1).astype(np.int32)
    X = PO.inputs(images, mask, side)
    v = np.where((mask > 0) & (images > 0), images.astype(np.float64), 0)
    v = v.reshape(2, 64, 2, 64, 2).sum((2, 4))
    want = np.log1p(v.reshape(2, -1) * 4096.0 / v.reshape(2, -1).sum(1, keepdims=True))
    np.testing.assert_allclose(X, want, rtol=1e-12)


def qmul(a, b):
    a0, a1, a2, a3 = a
    b0, b1, b2, b3 = b
    return np.array([a0 * b0 - a1 * b1 - a2 * b2 - a3 * b3, a0 * b1 + a1 * b0 + a2 * b3 - a3 * b2,
                     a0 * b2 - a1 * b3 + a2 * b0 + a3 * b1, a0 * b3 + a1 * b2 - a2 * b1 + a3 * b0])


def test_quarter_turn_is_a_turn_about_the_beam_axis():
    """The augmentation's claim: the pattern of rotation M Rz(-90 deg) is the
    pattern of M turned by one quarter (binned inputs), and its 6D label is
    (-c2, c1).  Trilinear slices of a smooth model at 128 x 128 pixels."""
    import emc_gb300 as E
    from emc_gb300 import synthetic as S
    from oracle import oracle as O
    side = 128
    x, y, z = E.calculate_coordinates(side, S.PIXEL_SIZE, S.DISTANCE, S.WAVELENGTH)
    g = np.arange(side) - side / 2 + 0.5
    zz, yy, xx = np.meshgrid(g, g, g, indexing="ij")
    model = (np.exp(-((xx - 9) ** 2 + (yy + 4) ** 2 + zz ** 2) / 90.0)
             + 0.6 * np.exp(-((xx + 12) ** 2 + (yy - 15) ** 2 + (zz - 6) ** 2) / 60.0)
             + 0.3 * np.exp(-(xx ** 2 + (yy - 2) ** 2 + (zz + 20) ** 2) / 200.0))
    rng = np.random.default_rng(8)
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    qz = np.array([np.sqrt(0.5), 0.0, 0.0, -np.sqrt(0.5)])  # Rz(-90 deg)
    q2 = qmul(q, qz)
    s1 = O.get_slices(model.ravel(), side, q[None], x, y, z, interp=1)
    s2 = O.get_slices(model.ravel(), side, q2[None], x, y, z, interp=1)
    mask = np.ones(side * side, np.int32)
    X1 = PO.inputs(s1 * 1000.0, mask, side)
    X2 = PO.inputs(s2 * 1000.0, mask, side)
    np.testing.assert_allclose(PO.turn(X1, 1), X2, rtol=1e-4, atol=1e-5)
    assert np.abs(PO.turn(X1, 1) - X1).max() > 0.1  # the pattern is not symmetric
    np.testing.assert_allclose(PO.turn_6d(PO.quat_to_6d(q), 1), PO.quat_to_6d(q2), atol=1e-12)
