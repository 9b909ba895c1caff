"""Python entry to the oracle (TEST INFRASTRUCTURE ONLY).

Loaded by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg; the
product never imports it.  Two oracles live here:

* `Ref*` / `ref_iteration`: the C restatement of the reference kernels in
  emc_oracle.c (quirk-exact: int-truncated scaling denominator, FP64 per-pixel
  likelihood, float host log-sum-exp, sequential float sums), composed the
  way main.cpp:239-480 composes the reference's cuda_* calls for one rank.
* `fused_iteration_fp64`: the semantics of the fused iteration (float
  scaling denominator, invalid pairs excluded, FP64 normaliser) evaluated
  entirely in FP64 with numpy GEMMs (the GEMM-decomposed form of
  emc_cuda.cu:196-216 and emc_atomic.cu:88-132).  Slicing reuses the C
  restatement so the voxel indices are the kernels' own.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"
_lib = None

f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
I, F, L = C.c_int, C.c_float, C.c_long


def lib():
    global _lib
    if _lib is None:
        if not LIB.exists():
            from .build import build
            build()
        l = C.CDLL(str(LIB))
        l.oracle_get_slices.argtypes = [f32p, I, f32p, f32p, f32p, f32p, f32p, I, I]
        l.oracle_update_scaling_full.argtypes = [f32p, f32p, i32p, f32p, I, I, I, I]
        l.oracle_calculate_responsabilities.argtypes = [f32p, f32p, i32p, F, f32p, f32p, f32p,
                                                        I, I, I, I, I]
        l.oracle_max_vector.argtypes = [f32p, I, I, f32p]
        l.oracle_respons_max_expf.argtypes = [f32p, f32p, I, I, f32p]
        l.oracle_normalize_respons.argtypes = [f32p, f32p, f32p, I, I, f32p]
        l.oracle_update_slices.argtypes = [f32p, f32p, i32p, f32p, f32p, i32p, I, I, I, I, f32p]
        l.oracle_insert_slices.argtypes = [f32p, i32p, f32p, f32p, f32p, f32p, f32p, I, I, f32p,
                                           f32p]
        l.oracle_divide_model.argtypes = [f32p, f32p, L]
        l.oracle_model_average.argtypes = [f32p, L]
        l.oracle_model_average.restype = F
        l.oracle_normalize_model.argtypes = [f32p, L]
        l.oracle_normalize_model.restype = F
        l.oracle_rot_matrix.argtypes = [f32p, f32p]
        i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
        l.oracle_nearest_voxels.argtypes = [f32p, I, f32p, f32p, f32p, I, I, I, i64p]
        l.oracle_trilinear_stencil.argtypes = [f32p, I, f32p, f32p, f32p, I, I, i64p, f32p]
        l.oracle_bin_images.argtypes = [f32p, i32p, I, I, I, I, I, f32p, i32p]
        l.oracle_normalize_images.argtypes = [f32p, i32p, C.c_void_p, I, I, f32p]
        l.oracle_mask_images.argtypes = [f32p, i32p, L]
        l.oracle_model_init_radial.argtypes = [f32p, I, I, I, f32p, f32p]
        l.oracle_model_init_orientations.argtypes = [f32p, i32p, I, I, f32p, f32p, f32p, f32p,
                                                     f32p, f32p]
        _lib = l
    return _lib


def _f(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _i(a):
    return np.ascontiguousarray(a, dtype=np.int32)


# ---------------------------------------------------------------- kernels --
def get_slices(model, side, rot, x, y, z, interp=0):
    R = rot.shape[0] if rot.ndim == 2 else rot.size // 4
    out = np.empty((R, side * side), np.float32)
    lib().oracle_get_slices(_f(model), side, out, _f(rot), _f(x), _f(y), _f(z), R, interp)
    return out


def update_scaling_full(images, slices, mask, scaling, start):
    n_images, n2 = images.shape
    chunk = slices.shape[0]
    lib().oracle_update_scaling_full(_f(images), _f(slices), _i(mask), scaling, n2, n_images,
                                     start, chunk)


def calculate_responsabilities(slices, images, mask, sigma, scaling, respons, weights, start,
                               diff=1):
    n_images, n2 = images.shape
    lib().oracle_calculate_responsabilities(_f(slices), _f(images), _i(mask), sigma, scaling,
                                            respons, _f(weights), n2, n_images, start,
                                            slices.shape[0], diff)


def max_vector(respons, n_images):
    out = np.empty(n_images, np.float32)
    lib().oracle_max_vector(_f(respons), n_images, respons.size // n_images, out)
    return out


def respons_max_expf(respons, maxv, n_images):
    out = np.empty(n_images, np.float32)
    lib().oracle_respons_max_expf(_f(respons), _f(maxv), n_images, respons.size // n_images, out)
    return out


def normalize_respons(respons, sums, maxv, n_images):
    lse = np.empty(n_images, np.float32)
    lib().oracle_normalize_respons(respons, _f(sums), _f(maxv), n_images,
                                   respons.size // n_images, lse)
    return lse


def update_slices(images, mask, respons, scaling, active, start, chunk):
    n_images, n2 = images.shape
    slices = np.empty((chunk, n2), np.float32)
    totals = np.empty(chunk, np.float32)
    lib().oracle_update_slices(_f(images), slices, _i(mask), _f(respons), _f(scaling), _i(active),
                               n_images, start, chunk, n2, totals)
    return slices, totals


def insert_slices(slices, mask, totals, rot_chunk, x, y, z, side, model, weight):
    lib().oracle_insert_slices(_f(slices), _i(mask), _f(totals), _f(rot_chunk), _f(x), _f(y),
                               _f(z), side, slices.shape[0], model, weight)


def divide_model(model, weight):
    lib().oracle_divide_model(model, _f(weight), model.size)


def model_average(model):
    return float(lib().oracle_model_average(_f(model), model.size))


def normalize_model(model):
    return float(lib().oracle_normalize_model(model, model.size))


def rot_matrix(q):
    m = np.empty(9, np.float32)
    lib().oracle_rot_matrix(_f(q), m)
    return m.reshape(3, 3)


# ------------------------------------------------- reference iteration -----
def sigma_at(iteration, sigma_start=0.4, sigma_final=0.12, half_life=25):
    """main.cpp:251 in the reference's precision (returned as float32)."""
    t = np.float32(-iteration / np.float32(half_life))
    return np.float32(sigma_final + (sigma_start - sigma_final) * np.exp(np.float64(t) * np.log(2.0)))


def ref_iteration(model, images, mask, x, y, z, quats, weights, sigma, side, chunk=5000, diff=1,
                  known_intensity=False, scaling_in=None):
    """One iteration of main.cpp:239-480 for one rank, through the C restatement.
    Returns dict(model, weight, respons, scaling, maxr, sums, lse)."""
    images = _f(images)
    n_images = images.shape[0]
    R = quats.shape[0]
    model = _f(model).copy()
    scaling = np.ones((R, n_images), np.float32) if scaling_in is None else _f(scaling_in).copy()
    respons = np.zeros((R, n_images), np.float32)
    if not known_intensity:
        for s0 in range(0, R, chunk):
            c = min(chunk, R - s0)
            sl = get_slices(model, side, quats[s0:s0 + c], x, y, z)
            update_scaling_full(images, sl, mask, scaling, s0)
    for s0 in range(0, R, chunk):
        c = min(chunk, R - s0)
        sl = get_slices(model, side, quats[s0:s0 + c], x, y, z)
        calculate_responsabilities(sl, images, mask, np.float32(sigma), scaling, respons, weights,
                                   s0, diff)
    L = respons.copy()
    maxr = max_vector(respons, n_images)
    sums = respons_max_expf(respons, maxr, n_images)
    lse = normalize_respons(respons, sums, maxr, n_images)
    active = np.ones(n_images, np.int32)
    new_model = np.zeros(side ** 3, np.float32)
    weight = np.zeros(side ** 3, np.float32)
    for s0 in range(0, R, chunk):
        c = min(chunk, R - s0)
        sl, tot = update_slices(images, mask, respons, scaling, active, s0, c)
        insert_slices(sl, mask, tot, quats[s0:s0 + c], x, y, z, side, new_model, weight)
    divide_model(new_model, weight)
    normalize_model(new_model)
    return dict(model=new_model, weight=weight, respons=respons, loglik=L, scaling=scaling,
                maxr=maxr, sums=sums, lse=lse)


# ------------------------------------------------ fused-path FP64 oracle ---
POIS_C = 0.02
SLICE_FLOOR = 1e-6


def _compact(mask):
    return np.nonzero(np.asarray(mask).reshape(-1))[0]


def nearest_voxels(quats, x, y, z, side, lo):
    """Voxel index per (rotation, pixel) with the kernels' float arithmetic,
    -1 outside [lo, side)."""
    R, P = quats.shape[0], np.asarray(x).size
    out = np.empty((R, P), np.int64)
    lib().oracle_nearest_voxels(_f(quats), R, _f(x), _f(y), _f(z), P, side, lo, out)
    return out


def trilinear_weights(quats, x, y, z, side):
    """(voxel index [R,P,8], weight [R,P,8]) of the trilinear stencil, weight 0
    outside the volume."""
    R, P = quats.shape[0], np.asarray(x).size
    vox = np.empty((R, P, 8), np.int64)
    wts = np.empty((R, P, 8), np.float32)
    lib().oracle_trilinear_stencil(_f(quats), R, _f(x), _f(y), _f(z), P, side, vox, wts)
    return vox, wts.astype(np.float64)


def fused_iteration_fp64(model, images, mask, x, y, z, quats, weights, sigma, side, diff=1,
                         interp=0, known_intensity=False, normalize_images=False, blur_sigma=0.0):
    """The fused iteration's semantics in FP64.  Returns dict(model, weight,
    respons [R,N], phi [R,N], loglik [R,N], lse [N], total_loglik)."""
    images = np.asarray(images, np.float64)
    N = images.shape[0]
    R = quats.shape[0]
    pix = _compact(mask)
    xs, ys, zs = _f(x)[pix], _f(y)[pix], _f(z)[pix]
    if normalize_images:
        c = (np.float32(side * side) / images[:, pix].astype(np.float32).sum(1, dtype=np.float32))
        K = (images[:, pix].astype(np.float32) * c.astype(np.float32)[:, None]).astype(np.float64)
    else:
        K = images[:, pix]
    # expand (the kernels' own float slices)
    S = get_slices(model, side, quats, x, y, z, interp)[:, pix].astype(np.float64)
    logw = np.log(np.asarray(weights, np.float64))
    valid_rot = (S > 0).sum(1)
    if diff == 1:
        Kt = np.where(K > 1e-10, K, 0.0)
        Mp = (S > 1e-10).astype(np.float64)
        if known_intensity:
            phi = np.ones((R, N))
            ok = np.ones((R, N), bool)
        else:
            num = Mp @ (Kt ** 2).T          # [R, N]
            den = (Mp * S) @ Kt.T
            ok = (num > 0) & (den > 0)
            phi = np.where(ok, num / np.where(ok, den, 1.0), 1.0)
        M = (S > 0).astype(np.float64)
        A = (M * S * S / (S + POIS_C)).sum(1)
        B = (M * S / (S + POIS_C)) @ K.T
        Cc = (M / (S + POIS_C)) @ (K ** 2).T
        Sig = A[:, None] - 2 * B / phi + Cc / phi ** 2
        ok &= valid_rot[:, None] > 0
        Lr = np.where(ok, logw[:, None] - Sig / (2.0 * np.maximum(valid_rot, 1)[:, None]
                                                 * float(sigma) ** 2), -np.inf)
    else:
        Sf = np.maximum(S, SLICE_FLOOR)
        Ksum = K.sum(1)
        Sr = Sf.sum(1)
        G = np.log(Sf) @ K.T
        if known_intensity:
            phi = np.ones((R, N))
            Lr = logw[:, None] + G - Sr[:, None]
        else:
            with np.errstate(divide="ignore", invalid="ignore"):
                phi = np.where(Ksum[None, :] > 0, Ksum[None, :] / Sr[:, None], 0.0)
                Lr = np.where(Ksum[None, :] > 0,
                              logw[:, None] + G + Ksum[None, :] * np.log(np.where(phi > 0, phi, 1.0))
                              - Ksum[None, :], logw[:, None])
    Mx = Lr.max(0)
    with np.errstate(invalid="ignore"):
        lse = np.where(np.isfinite(Mx), Mx + np.log(np.exp(Lr - Mx[None, :]).sum(0)), np.inf)
        P = np.where(np.isfinite(lse)[None, :], np.exp(Lr - lse[None, :]), 0.0)
    P = np.nan_to_num(P)
    m = mstep_fp64(P, phi, K, xs, ys, zs, quats, side, interp, blur_sigma)
    total_ll = float(lse[np.isfinite(lse)].sum())
    return dict(model=m["model"], weight=m["weight"], respons=P, phi=phi, loglik=Lr, lse=lse,
                total_loglik=total_ll, T=m["T"], mean_before=m["mean_before"])


def compacted_counts(images, mask, side, normalize_images=False):
    """The M-step's pattern operand: counts at the mask pixels (times the
    reference's per-pattern factor when normalising), FP64 [N, P_eff]."""
    images = np.asarray(images, np.float64)
    pix = _compact(mask)
    if normalize_images:
        c = (np.float32(side * side) / images[:, pix].astype(np.float32).sum(1, dtype=np.float32))
        return (images[:, pix].astype(np.float32) * c.astype(np.float32)[:, None]).astype(np.float64)
    return images[:, pix]


def mstep_fp64(P, phi, K, xs, ys, zs, quats, side, interp=0, blur_sigma=0.0):
    """M-step of the fused iteration from given responsibilities P [R, N] and
    scaling phi [R, N]: U = (P/phi) K, insertion of T_r (U/T_r) with weight
    T_r (rotations with T_r > 1e-10), divide, normalise to mean 1, blur."""
    P = np.asarray(P, np.float64)
    phi = np.asarray(phi, np.float64)
    with np.errstate(divide="ignore", invalid="ignore"):
        Qm = np.where(phi > 0, P / np.where(phi > 0, phi, 1.0), 0.0)
    # T_r is summed in FP64 and kept as a float, and the live test is the
    # float comparison T_r > 1e-10f, exactly as in the kernels (a rotation
    # whose total sits at the threshold must decide the same way)
    T32 = P.sum(1).astype(np.float32)
    T = T32.astype(np.float64)
    U = Qm @ K  # [R, P_eff]
    n3 = side ** 3
    new_m = np.zeros(n3)
    new_w = np.zeros(n3)
    live = T32 > np.float32(1e-10)
    if interp == 0:
        vox = nearest_voxels(quats, xs, ys, zs, side, 0)
        sel = (vox >= 0) & live[:, None]
        new_m += np.bincount(vox[sel], weights=U[sel], minlength=n3)
        new_w += np.bincount(vox[sel], weights=np.broadcast_to(T[:, None], U.shape)[sel],
                             minlength=n3)
    else:
        vox, wts = trilinear_weights(quats, xs, ys, zs, side)
        wts = wts * live[:, None, None]
        new_m += np.bincount(vox.reshape(-1), weights=(U[:, :, None] * wts).reshape(-1),
                             minlength=n3)
        new_w += np.bincount(vox.reshape(-1), weights=(T[:, None, None] * wts).reshape(-1),
                             minlength=n3)
    out = np.where(new_w > 0, new_m / np.where(new_w > 0, new_w, 1.0), -1.0)
    pos = out > 0
    mean = out[pos].mean() if pos.any() else 0.0
    out = out * (1.0 / mean)
    if blur_sigma > 0:
        out = blur_fft_fp64(out, side, blur_sigma)
    return dict(model=out, weight=new_w, T=T, mean_before=mean)


def blur_fft_fp64(model, side, sigma):
    """emc_cuda.cu:1404-1492 as intended: negative voxels masked to 0, the
    spectrum multiplied by exp(-2 pi^2 sigma^2 |k|^2 / s^2) (folded k), masked
    voxels restored to -1.  FP64 FFT."""
    v = np.asarray(model, np.float64).reshape(side, side, side)
    keep = ~(v < 0)
    v = np.where(keep, v, 0.0)
    k = np.arange(side)
    kf = np.minimum(k, side - k).astype(np.float64)
    m1 = np.exp(-2 * np.pi ** 2 * sigma ** 2 * kf ** 2 / side ** 2)
    Mul = m1[:, None, None] * m1[None, :, None] * m1[None, None, :]
    out = np.fft.ifftn(np.fft.fftn(v) * Mul).real
    return np.where(keep, out, -1.0).reshape(-1)


# ------------------------------------------------------ preprocessing ----
def bin_images(raw, raw_mask, side, stride):
    """read_images binning (emc_helper.cpp:226-243): raw [n, h, w] -> (images [n, side*side],
    masks [n, side*side])."""
    raw, raw_mask = _f(raw), _i(raw_mask)
    n, h, w = raw.shape
    images = np.zeros((n, side * side), np.float32)
    masks = np.zeros((n, side * side), np.int32)
    lib().oracle_bin_images(raw, raw_mask, w, h, n, side, stride, images, masks)
    return images, masks


def normalize_images(images, mask, masks=None):
    """normalize_images_central_part / _individual_mask (emc_helper.cpp:389-438)."""
    out = _f(images).copy()
    n, n2 = out.shape
    fac = np.zeros(n, np.float32)
    mk = None if masks is None else _i(masks)
    lib().oracle_normalize_images(out, _i(mask), None if mk is None else mk.ctypes.data, n2, n,
                                  fac)
    return out, fac


def mask_images(images, masks):
    out = _f(images).copy()
    lib().oracle_mask_images(out, _i(masks), out.size)
    return out


def model_init_radial(images, side, float_sums=True):
    """model_init, model_input 3 (emc_helper.cpp:458-502); float_sums=True is the
    reference's sequential float ring sums, False FP64 ring sums."""
    images = _f(images)
    radavg = np.zeros(side // 2 + 1, np.float32)
    model = np.zeros(side ** 3, np.float32)
    lib().oracle_model_init_radial(images, images.shape[0], side, int(float_sums), radavg, model)
    return model, radavg


def model_init_orientations(images, mask, side, quats, x, y, z):
    """model_init, model_input 1 (emc_helper.cpp:503-518) at the given quaternions."""
    images = _f(images)
    model = np.zeros(side ** 3, np.float32)
    weight = np.zeros(side ** 3, np.float32)
    lib().oracle_model_init_orientations(images, _i(mask), images.shape[0], side, _f(quats),
                                         _f(x), _f(y), _f(z), model, weight)
    return model, weight


# ------------------------------------- the reference's own host code ----
def ref_rotations(n):
    """(quats [R, 4], weights [R]) float32 from the reference's own
    generate_rotation_list (rotations.c:77-458, oracle/_ref/ref_rotations
    built by build_ref.sh), or None when that build is absent."""
    import subprocess
    import tempfile
    exe = HERE / "_ref" / "ref_rotations"
    if not exe.exists():
        return None
    with tempfile.TemporaryDirectory() as d:  # it also writes debug_samples.data there
        subprocess.run([str(exe), str(int(n)), f"{d}/rot.bin"], cwd=d, check=True,
                       capture_output=True)
        b = open(f"{d}/rot.bin", "rb").read()
    R = int(np.frombuffer(b[:4], np.int32)[0])
    q = np.frombuffer(b[4:4 + 16 * R], np.float32).reshape(R, 4).copy()
    w = np.frombuffer(b[4 + 16 * R:4 + 20 * R], np.float32).copy()
    return q, w


def ref_coordinates(side, pixel_size, detector_distance, wavelength):
    """(x, y, z) float32 [side*side] from the reference's own
    calculate_coordinates (emc_helper.cpp:55-79 behind
    oracle/ref_helper_harness.cpp), or None when that build is absent."""
    from .build import ref_helper
    h = ref_helper()
    if h is None:
        return None
    out = [np.zeros(side * side, np.float32) for _ in range(3)]
    h.refh_calculate_coordinates(side, pixel_size, detector_distance, wavelength,
                                 *[a.ctypes.data_as(C.c_void_p) for a in out])
    return tuple(out)
