"""emc_gb300 -- GB300-native (sm_103a) EMC iteration behind the reference's
`cuda_*` interface.

Python mirror of the C ABI in include/emc_gb300.h.  `Context` exposes the
reference's per-function entry points under their reference names
(emc_cuda_help.h:9-117): get_slices, update_scaling_full,
calculate_responsabilities, max_vector, respons_max_expf,
norm_respons_sumexpf, update_slices, divide_model_by_weight,
normalize_model, model_max, model_average, blur_model, reset_real.  Buffers are
torch CUDA tensors (device memory and streams only -- every computation is a
kernel of libemc_gb300.so).  `Plan` drives the fused iteration.

Errors: every call checks the int status and raises EmcError with the
context's last error text, where the reference printed and continued.
"""
from __future__ import annotations

import atexit
import ctypes as C
import weakref

import numpy as np

from . import _lib
from ._lib import (DIFF_ABSOLUTE, DIFF_POISSON, DIFF_RELATIVE, DIFF_TRUE_POISSON,  # noqa: F401
                   INSERT_ATOMIC, INSERT_DETERMINISTIC, INSERT_SORTED, INTERP_NEAREST,
                   INTERP_TRILINEAR,
                   PREC_FP32, PREC_MIXED, EmcError, IterStats, PlanDesc)

__all__ = [
    "Context", "Plan", "Batch", "EmcError", "generate_rotations", "rotation_count",
    "calculate_coordinates", "sigma_schedule", "library",
]


def library():
    return _lib.load()


def _ptr(t, dtype=None, name="buffer"):
    """Raw device pointer of a contiguous CUDA tensor (None -> NULL)."""
    if t is None:
        return None
    if isinstance(t, int):
        return t
    if not t.is_cuda:
        raise EmcError(f"{name} must be a CUDA tensor")
    if not t.is_contiguous():
        raise EmcError(f"{name} must be contiguous")
    if dtype is not None and t.dtype != dtype:
        raise EmcError(f"{name} must be {dtype}, got {t.dtype}")
    return t.data_ptr()


def rotation_count(n: int) -> int:
    return int(_lib.load().emc_rotation_count(n))


def generate_rotations(n: int):
    """600-cell sampling at level n (rotations.c:77-458): (quats [R,4], weights [R])."""
    lib = _lib.load()
    R = lib.emc_rotation_count(n)
    if R <= 0:
        raise EmcError(f"bad rotation level {n}")
    q = np.zeros((R, 4), np.float32)
    w = np.zeros(R, np.float32)
    rc = lib.emc_generate_rotations(n, q.ctypes.data, w.ctypes.data, R)
    if rc != R:
        raise EmcError(f"emc_generate_rotations({n}) returned {rc}")
    return q, w


def calculate_coordinates(side: int, pixel_size: float, detector_distance: float,
                          wavelength: float):
    """Detector pixel coordinates (emc_helper.cpp:55-79): x, y, z as [side*side] float32."""
    lib = _lib.load()
    x = np.zeros(side * side, np.float32)
    y = np.zeros_like(x)
    z = np.zeros_like(x)
    rc = lib.emc_calculate_coordinates(side, pixel_size, detector_distance, wavelength,
                                       x.ctypes.data, y.ctypes.data, z.ctypes.data)
    if rc != 0:
        raise EmcError(f"emc_calculate_coordinates failed ({rc})")
    return x, y, z


def sigma_schedule(iteration: int, sigma_start: float, sigma_final: float, half_life: int) -> float:
    return float(_lib.load().emc_sigma_schedule(iteration, sigma_start, sigma_final, half_life))


def random_rotations(seed: int, n: int):
    """quaternion_random (rotations.c:30-41) n times from a seeded generator: [n, 4] float32."""
    q = np.zeros((n, 4), np.float32)
    rc = _lib.load().emc_random_rotations(int(seed), int(n), q.ctypes.data if n else None)
    if rc != 0:
        raise EmcError(f"emc_random_rotations failed ({rc})")
    return q


def read_config(path=None, text=None) -> "_lib.Config":
    """emc.conf (configs.cpp:40-90 keys) -> emc_config; raises EmcError on a
    syntax or type error."""
    lib = _lib.load()
    cfg = _lib.Config()
    err = C.create_string_buffer(512)
    if text is not None:
        lib.emc_config_defaults(C.byref(cfg))
        rc = lib.emc_config_parse(text.encode(), C.byref(cfg), err, 512)
    else:
        rc = lib.emc_config_read(str(path).encode(), C.byref(cfg), err, 512)
    if rc != 0:
        raise EmcError(f"config: {err.value.decode()}")
    return cfg


_LIVE_CONTEXTS = weakref.WeakSet()


@atexit.register
def _close_all():
    """Destroy what is still open while the CUDA runtime is alive: at
    interpreter exit objects are otherwise collected in no particular order,
    after the runtime's own teardown may have begun."""
    for ctx in list(_LIVE_CONTEXTS):
        try:
            ctx.close()
        except Exception:
            pass


def _stream_ordered(fn):
    """Orders a library call against torch's current stream both ways: the
    context's stream waits for work already queued on torch's current stream
    (e.g. the kernel that filled an input tensor), and torch's current stream
    waits for the library's kernels before any later torch work reads their
    outputs.  A no-op when the two streams are the same."""
    import functools

    @functools.wraps(fn)
    def run(self, *a, **k):
        ctx = self if isinstance(self, Context) else self.ctx
        if not getattr(ctx, "_h", None):
            return fn(self, *a, **k)
        import torch
        cur = torch.cuda.current_stream(ctx.device)
        handle = ctx.stream
        if handle == cur.cuda_stream:
            return fn(self, *a, **k)
        mine = ctx._ext_stream(handle)
        mine.wait_stream(cur)
        try:
            return fn(self, *a, **k)
        finally:
            cur.wait_stream(mine)
    return run


class Context:
    """One device, one stream (replaces cuda_set_device, emc_cuda.cu:867-870).

    Calls taking torch tensors are ordered against torch's current stream
    (see _stream_ordered), so tensors written by torch before a call and read
    by torch after it need no explicit synchronisation."""

    def __init__(self, device: int = 0):
        self._lib = _lib.load()
        h = C.c_void_p()
        rc = self._lib.emc_ctx_create(C.byref(h), device)
        if rc != 0:
            raise EmcError(f"emc_ctx_create(device={device}) failed: {_lib.ERRORS.get(rc, rc)}")
        self._h = h
        self.device = device
        self._children = weakref.WeakSet()  # plans and batches, closed before the context
        _LIVE_CONTEXTS.add(self)

    # -- plumbing ------------------------------------------------------------
    @property
    def handle(self):
        return self._h

    def _check(self, rc, what):
        if rc != 0:
            msg = self._lib.emc_last_error(self._h).decode()
            raise EmcError(f"{what}: {_lib.ERRORS.get(rc, rc)}: {msg}")

    def close(self):
        if getattr(self, "_h", None):
            kids = list(getattr(self, "_children", ()))
            for child in sorted(kids, key=lambda c: not isinstance(c, Batch)):  # batches first
                child.close()
            self._lib.emc_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream=None):
        self._check(self._lib.emc_set_stream(self._h, stream), "set_stream")

    def _ext_stream(self, handle):
        """torch view of the library stream `handle` (cached per handle)."""
        import torch
        cache = self.__dict__.setdefault("_ext_streams", {})
        st = cache.get(handle)
        if st is None:
            st = cache[handle] = torch.cuda.ExternalStream(handle, device=self.device)
        return st

    @property
    def stream(self) -> int:
        return self._lib.emc_get_stream(self._h) or 0

    def sync(self):
        self._check(self._lib.emc_sync(self._h), "sync")

    @property
    def kernel_launches(self) -> int:
        return int(self._lib.emc_kernel_launches(self._h))

    # -- reference entry points ---------------------------------------------
    def get_slices(self, model, side, slices, rot, x, y, z, start, chunk, interp=INTERP_NEAREST):
        import torch
        self._check(self._lib.emc_get_slices(
            self._h, _ptr(model, torch.float32, "model"), side, _ptr(slices, torch.float32, "slices"),
            _ptr(rot, torch.float32, "rot"), _ptr(x), _ptr(y), _ptr(z), start, chunk, interp),
            "get_slices")

    def update_scaling_full(self, images, slices, mask, scaling, n_2d, n_images, start, chunk,
                            diff=DIFF_POISSON):
        import torch
        self._check(self._lib.emc_update_scaling_full(
            self._h, _ptr(images, torch.float32), _ptr(slices, torch.float32),
            _ptr(mask, torch.int32, "mask"), _ptr(scaling, torch.float32), n_2d, n_images, start,
            chunk, diff), "update_scaling_full")

    def calculate_responsabilities(self, slices, images, mask, sigma, scaling, respons, weights,
                                   n_2d, n_images, start, chunk, diff=DIFF_POISSON):
        import torch
        self._check(self._lib.emc_calculate_responsabilities(
            self._h, _ptr(slices, torch.float32), _ptr(images, torch.float32),
            _ptr(mask, torch.int32), float(sigma), _ptr(scaling, torch.float32),
            _ptr(respons, torch.float32), _ptr(weights, torch.float32), n_2d, n_images, start,
            chunk, diff), "calculate_responsabilities")

    def max_vector(self, respons, n_images, n_slices, maxr):
        self._check(self._lib.emc_max_vector(self._h, _ptr(respons), n_images, n_slices,
                                             _ptr(maxr)), "max_vector")

    def respons_max_expf(self, respons, maxv, n_images, n_slices, out_sum):
        self._check(self._lib.emc_respons_max_expf(self._h, _ptr(respons), _ptr(maxv), n_images,
                                                   n_slices, _ptr(out_sum)), "respons_max_expf")

    def norm_respons_sumexpf(self, respons, lse, maxv, n_images, n_slices):
        self._check(self._lib.emc_norm_respons_sumexpf(self._h, _ptr(respons), _ptr(lse),
                                                       _ptr(maxv), n_images, n_slices),
                    "norm_respons_sumexpf")

    def log_sum_max(self, out_sum, maxv, lse, n_images):
        self._check(self._lib.emc_log_sum_max(self._h, _ptr(out_sum), _ptr(maxv), _ptr(lse),
                                              n_images), "log_sum_max")

    def update_slices(self, images, slices, mask, respons, scaling, active, n_images, start,
                      chunk, n_2d, side, model, x, y, z, rot_chunk, weight):
        import torch
        self._check(self._lib.emc_update_slices(
            self._h, _ptr(images), _ptr(slices), _ptr(mask, torch.int32), _ptr(respons),
            _ptr(scaling), _ptr(active, torch.int32, "active"), n_images, start, chunk, n_2d, side,
            _ptr(model), _ptr(x), _ptr(y), _ptr(z), _ptr(rot_chunk), _ptr(weight)),
            "update_slices")

    def divide_model_by_weight(self, side, model, weight):
        self._check(self._lib.emc_divide_model_by_weight(self._h, side, _ptr(model), _ptr(weight)),
                    "divide_model_by_weight")

    def normalize_model(self, side, model) -> float:
        m = C.c_float()
        self._check(self._lib.emc_normalize_model(self._h, side, _ptr(model), C.byref(m)),
                    "normalize_model")
        return float(m.value)

    def model_max(self, model, n=None) -> float:
        m = C.c_float()
        self._check(self._lib.emc_model_max(self._h, _ptr(model), n or model.numel(), C.byref(m)),
                    "model_max")
        return float(m.value)

    def model_average(self, model, n=None) -> float:
        m = C.c_float()
        self._check(self._lib.emc_model_average(self._h, _ptr(model), n or model.numel(),
                                                C.byref(m)), "model_average")
        return float(m.value)

    def blur_model(self, model, side, sigma):
        self._check(self._lib.emc_blur_model(self._h, _ptr(model), side, float(sigma)),
                    "blur_model")

    # -- preprocessing and model initialisation (main.cpp:92-108) -----------
    def bin_images(self, raw, raw_mask, raw_w, raw_h, n_images, side, stride, images, masks):
        import torch
        self._check(self._lib.emc_bin_images(
            self._h, _ptr(raw, torch.float32, "raw"), _ptr(raw_mask, torch.int32, "raw_mask"),
            raw_w, raw_h, n_images, side, stride, _ptr(images, torch.float32, "images"),
            _ptr(masks, torch.int32, "masks")), "bin_images")

    def normalize_images(self, images, mask, n_2d, n_images, masks=None):
        import torch
        self._check(self._lib.emc_normalize_images(
            self._h, _ptr(images, torch.float32, "images"), _ptr(mask, torch.int32, "mask"),
            _ptr(masks, torch.int32, "masks"), n_2d, n_images), "normalize_images")

    def mask_model(self, images, masks, n_2d, n_images):
        import torch
        self._check(self._lib.emc_mask_images(self._h, _ptr(images, torch.float32, "images"),
                                              _ptr(masks, torch.int32, "masks"), n_2d,
                                              n_images), "mask_images")

    def model_init_radial(self, images, n_images, side, model):
        import torch
        self._check(self._lib.emc_model_init_radial(
            self._h, _ptr(images, torch.float32, "images"), n_images, side,
            _ptr(model, torch.float32, "model")), "model_init_radial")

    def model_init_orientations(self, images, mask, n_images, side, rot, x, y, z, model, weight):
        import torch
        self._check(self._lib.emc_model_init_orientations(
            self._h, _ptr(images, torch.float32, "images"), _ptr(mask, torch.int32, "mask"),
            n_images, side, _ptr(rot, torch.float32, "rot"), _ptr(x), _ptr(y), _ptr(z),
            _ptr(model, torch.float32, "model"), _ptr(weight, torch.float32, "weight")),
            "model_init_orientations")

    def reset_real(self, x, n=None):
        self._check(self._lib.emc_reset_real(self._h, _ptr(x), n if n is not None else x.numel()),
                    "reset_real")

    def copy_real_d2d(self, dst, src_ptr: int, start: int = 0, n=None):
        """dst[start:start+n] = n floats at device address src_ptr."""
        n = dst.numel() - start if n is None else n
        self._check(self._lib.emc_copy_real_d2d(self._h, _ptr(dst), src_ptr, start, n),
                    "copy_real_d2d")

    def copy_real_to_host(self, src_ptr: int, n: int) -> np.ndarray:
        out = np.empty(n, np.float32)
        self._check(self._lib.emc_copy_real_to_host(self._h, out.ctypes.data, src_ptr, n),
                    "copy_real_to_host")
        return out


class Plan:
    """Fused EMC iteration (emc_plan_* in the C ABI)."""

    def __init__(self, ctx: Context, side, n_images, n_rot, diff=DIFF_POISSON,
                 interp=INTERP_NEAREST, precision=PREC_FP32, insert_mode=INSERT_ATOMIC,
                 known_intensity=0, normalize_images=0, blur_sigma=0.0):
        self.ctx = ctx
        self._lib = ctx._lib
        d = PlanDesc(side, n_images, n_rot, diff, interp, precision, insert_mode,
                     known_intensity, normalize_images, float(blur_sigma))
        self.desc = d
        h = C.c_void_p()
        ctx._check(self._lib.emc_plan_create(ctx.handle, C.byref(d), C.byref(h)), "plan_create")
        self._h = h
        self._bound = None
        ctx._children.add(self)

    @property
    def workspace_bytes(self) -> int:
        return int(self._lib.emc_plan_workspace_bytes(self._h))

    def bind(self, images, mask, x, y, z, rot, rot_weights):
        import torch
        self._bound = (images, mask, x, y, z, rot, rot_weights)  # keep alive
        self.ctx._check(self._lib.emc_plan_bind(
            self._h, _ptr(images, torch.float32, "images"), _ptr(mask, torch.int32, "mask"),
            _ptr(x), _ptr(y), _ptr(z), _ptr(rot, torch.float32, "rot"),
            _ptr(rot_weights, torch.float32, "rot_weights")), "plan_bind")

    def iterate(self, model, weight, sigma, stats: bool = True):
        st = IterStats()
        self.ctx._check(self._lib.emc_iterate(self._h, _ptr(model), _ptr(weight), float(sigma),
                                              C.byref(st) if stats else None), "iterate")
        return st if stats else None

    def set_pruning(self, on: bool = True, min_mass: float = 0.999, dilate: float = 1.0,
                    full_every: int = 0):
        """Pruned iterations (tensor-core path): see emc_plan_set_pruning."""
        self.ctx._check(self._lib.emc_plan_set_pruning(self._h, int(on), float(min_mass),
                                                       float(dilate), int(full_every)),
                        "plan_set_pruning")

    def prune_info(self) -> dict:
        info = _lib.PruneInfo()
        self.ctx._check(self._lib.emc_plan_prune_info(self._h, C.byref(info)), "plan_prune_info")
        return {k: getattr(info, k) for k, _ in info._fields_}

    def pattern_order(self):
        """Input pattern index of each position of the last iteration's results."""
        out = np.zeros(self.desc.n_images, np.int32)
        self.ctx._check(self._lib.emc_plan_pattern_order(self._h, out.ctypes.data),
                        "plan_pattern_order")
        return out

    def best_quaternions(self, out):
        """The most probable rotation of every pattern in the last
        iteration's responsibilities: out [N][4] float32 CUDA tensor, input
        pattern order (emc_plan_best_quaternions)."""
        self.ctx._check(self._lib.emc_plan_best_quaternions(self._h, _ptr(out, name="out")),
                        "plan_best_quaternions")
        return out

    def set_proposals(self, quats, fraction: float = 0.02, probe_stride: int = 16):
        """Seeds the next pruned iteration from rotation proposals quats
        [N][modes][4] (emc_plan_set_proposals)."""
        if quats.dim() != 3 or quats.shape[2] != 4 or quats.shape[0] != self.desc.n_images:
            raise EmcError("proposals must be [n_images][modes][4]")
        self.ctx._check(self._lib.emc_plan_set_proposals(
            self._h, _ptr(quats, name="quats"), int(quats.shape[1]), float(fraction),
            int(probe_stride)), "plan_set_proposals")

    def rotation_order(self):
        """Input rotation index of each row of the last iteration's results."""
        out = np.zeros(self.desc.n_rot, np.int32)
        self.ctx._check(self._lib.emc_plan_rotation_order(self._h, out.ctypes.data),
                        "plan_rotation_order")
        return out

    def iterate_async(self, model, weight, sigma):
        """Enqueue one iteration; errors and stats come from wait()."""
        self.ctx._check(self._lib.emc_iterate_async(self._h, _ptr(model), _ptr(weight),
                                                    float(sigma)), "iterate_async")

    def wait(self, stats: bool = True):
        st = IterStats()
        self.ctx._check(self._lib.emc_plan_wait(self._h, C.byref(st) if stats else None),
                        "plan_wait")
        return st if stats else None

    def capture(self, model, weight):
        """Record one iteration on (model, weight) into a CUDA graph."""
        self._captured = (model, weight)  # keep alive
        self.ctx._check(self._lib.emc_plan_capture(self._h, _ptr(model), _ptr(weight)),
                        "plan_capture")

    def replay(self, sigma):
        """One iteration in place on the captured buffers (asynchronous)."""
        self.ctx._check(self._lib.emc_plan_replay(self._h, float(sigma)), "plan_replay")

    PHASES = ("expand", "estep", "lse", "mprep", "mstep", "finish")
    OPT_ESTEP_GHLO = 3
    OPT_MSTEP_QLO = 2
    OPT_MSTEP_AGGREGATE = 4
    OPT_COUNTS_ROUND = 5
    OPT_ESTEP_RASTER = 6
    OPT_ESTEP_PAIR = 7
    OPT_MSTEP_RASTER = 8
    OPT_DEBUG_SPIN = 9
    OPT_MSTEP_PAIR = 10
    OPT_GLO_TAIL = 11

    def set_option(self, option: int, value: int):
        self.ctx._check(self._lib.emc_plan_set_option(self._h, option, value), "plan_set_option")

    def get_option(self, option: int) -> int:
        v = C.c_int(0)
        self.ctx._check(self._lib.emc_plan_get_option(self._h, option, C.byref(v)),
                        "plan_get_option")
        return v.value

    def autotune(self, model, sigma: float = 0.4) -> tuple:
        """Picks the likelihood kernel's tile order (OPT_ESTEP_RASTER) by
        timing the candidates on `model` (emc_plan_autotune).  Returns
        (raster, ms of the timed prefix); (0, 0.0) for FP32 plans."""
        import ctypes as C
        r, ms = C.c_int(0), C.c_float(0.0)
        self.ctx._check(self._lib.emc_plan_autotune(self._h, _ptr(model, name="model"),
                                                    float(sigma), C.byref(r), C.byref(ms)),
                        "plan_autotune")
        return r.value, ms.value

    def time_likelihood(self, raster: int, first: int = 0, count: int = 1 << 30,
                        model=None, sigma: float = 0.4) -> tuple:
        """One timed launch of the likelihood kernel over tiles [first,
        first + count) of order `raster` (emc_plan_time_likelihood); model
        given: expanded first.  Returns (ms, tiles in the full grid)."""
        import ctypes as C
        ms, tot = C.c_float(0.0), C.c_int(0)
        self.ctx._check(self._lib.emc_plan_time_likelihood(
            self._h, _ptr(model, name="model"), float(sigma), int(raster), int(first),
            int(count), C.byref(ms), C.byref(tot)), "plan_time_likelihood")
        return ms.value, tot.value

    def set_profiling(self, on: bool = True):
        self.ctx._check(self._lib.emc_plan_set_profiling(self._h, int(on)), "plan_set_profiling")

    def phase_ms(self) -> dict:
        """Per-phase durations (ms) of the last iteration, from CUDA events
        recorded on the context stream."""
        out = (C.c_float * 6)()
        self.ctx._check(self._lib.emc_plan_phase_ms(self._h, out, 6), "plan_phase_ms")
        return dict(zip(self.PHASES, [float(v) for v in out]))

    # -- one rank of a rotation split (emc_rank_*) ----------------------------
    def rank_estep(self, model, sigma, d_max, d_sumexp):
        """Expand + likelihood over this plan's rotations; d_max [N] float32
        and d_sumexp [N] float64 receive the per-pattern partials."""
        import torch
        self.ctx._check(self._lib.emc_rank_estep(
            self._h, _ptr(model, torch.float32, "model"), float(sigma),
            _ptr(d_max, torch.float32, "d_max"), _ptr(d_sumexp, torch.float64, "d_sumexp")),
            "rank_estep")

    def rank_mstep(self, lse, model_sum, weight_sum):
        """M-step of this plan's rotations with the global lse [N] float64;
        writes the un-normalised sums."""
        import torch
        self.ctx._check(self._lib.emc_rank_mstep(
            self._h, _ptr(lse, torch.float64, "lse"), _ptr(model_sum, torch.float32, "model_sum"),
            _ptr(weight_sum, torch.float32, "weight_sum")), "rank_mstep")

    def model_from_sums(self, model_sum, weight_sum, n_ranks, model, weight):
        import torch
        self.ctx._check(self._lib.emc_model_from_sums(
            self._h, _ptr(model_sum, torch.float32), _ptr(weight_sum, torch.float32),
            int(n_ranks), _ptr(model, torch.float32, "model"),
            _ptr(weight, torch.float32, "weight")), "model_from_sums")

    def results(self):
        r, s, l = C.c_void_p(), C.c_void_p(), C.c_void_p()
        self.ctx._check(self._lib.emc_plan_results(self._h, C.byref(r), C.byref(s), C.byref(l)),
                        "plan_results")
        return r.value, s.value, l.value

    def close(self):
        if getattr(self, "_h", None):
            self._lib.emc_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Proposal:
    """The learned rotation proposal network (emc_proposal_* in the C ABI):
    trained on the GPU on EMC's most probable rotations, it predicts each
    pattern's rotation and its Friedel mate."""

    def __init__(self, ctx: Context, seed: int = 0):
        self.ctx = ctx
        self._lib = ctx._lib
        h = C.c_void_p()
        ctx._check(self._lib.emc_proposal_create(ctx._h, int(seed), C.byref(h)), "proposal_create")
        self._h = h
        self.n_params = int(self._lib.emc_proposal_param_count(h))
        self.n_data = 0
        ctx._children.add(self)

    def params(self) -> np.ndarray:
        out = np.empty(self.n_params, np.float32)
        self.ctx._check(self._lib.emc_proposal_params(self._h, out.ctypes.data, 1),
                        "proposal_params")
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        if p.size != self.n_params:
            raise EmcError(f"expected {self.n_params} parameters")
        self.ctx._check(self._lib.emc_proposal_params(self._h, p.ctypes.data, 0),
                        "proposal_params")

    def set_data(self, images, mask, side: int, fit_stats: bool = True):
        """Bins the patterns images [N][side^2] (mask [side^2] int32) into
        the network's input rows, standardised per input pixel with
        statistics fitted on these patterns (fit_stats) or the stored ones."""
        n = images.shape[0]
        self.ctx._check(self._lib.emc_proposal_set_data(
            self._h, _ptr(images, name="images"), _ptr(mask, name="mask"), int(side), int(n),
            int(bool(fit_stats))), "proposal_set_data")
        self.n_data = n

    def stats(self) -> np.ndarray:
        """Input statistics [2][4096]: per-pixel mean and 1 / spread."""
        out = np.empty((2, 4096), np.float32)
        self.ctx._check(self._lib.emc_proposal_stats(self._h, out.ctypes.data, 1),
                        "proposal_stats")
        return out

    def inputs(self, first: int, count: int) -> np.ndarray:
        out = np.empty((count, 4096), np.float32)
        self.ctx._check(self._lib.emc_proposal_inputs(self._h, int(first), int(count),
                                                      out.ctypes.data), "proposal_inputs")
        return out

    def loss_grad(self, rows, quats):
        """Mean loss and parameter gradient of one batch (rows of the data,
        labels quats [N][4] CUDA float32)."""
        rows = np.ascontiguousarray(rows, np.int32)
        loss = C.c_float(0.0)
        g = np.empty(self.n_params, np.float32)
        self.ctx._check(self._lib.emc_proposal_loss_grad(
            self._h, rows.ctypes.data, int(rows.size), _ptr(quats, name="quats"), C.byref(loss),
            g.ctypes.data), "proposal_loss_grad")
        return loss.value, g

    def train(self, quats, rows=None, epochs: int = 10, batch: int = 256, lr: float = 1e-3,
              seed: int = 0, augment: bool = True) -> np.ndarray:
        """Adam over shuffled minibatches (augment: random in-plane quarter
        turns); returns each epoch's mean loss."""
        losses = np.zeros(max(epochs, 1), np.float32)
        if rows is None:
            rp, nr = None, 0
        else:
            rows = np.ascontiguousarray(rows, np.int32)
            rp, nr = rows.ctypes.data, int(rows.size)
        self.ctx._check(self._lib.emc_proposal_train(
            self._h, _ptr(quats, name="quats"), rp, nr, int(epochs), int(batch), float(lr),
            int(seed), int(bool(augment)), losses.ctypes.data), "proposal_train")
        return losses[:epochs]

    def predict(self, out):
        """out [N][2][4] CUDA float32: each pattern's predicted rotation and
        its Friedel mate (quaternions, w >= 0)."""
        self.ctx._check(self._lib.emc_proposal_predict(self._h, _ptr(out, name="out")),
                        "proposal_predict")
        return out

    def close(self):
        if getattr(self, "_h", None):
            self._lib.emc_proposal_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Independent reconstructions run together: one graph launch per
    iteration covers every plan (emc_batch_* in the C ABI)."""

    def __init__(self, plans, models, weights):
        n = len(plans)
        self.plans = list(plans)
        self._keep = (list(models), list(weights))
        self._lib = plans[0]._lib
        hp = (C.c_void_p * n)(*[p._h.value for p in plans])
        hm = (C.c_void_p * n)(*[_ptr(m) for m in models])
        hw = (C.c_void_p * n)(*[_ptr(w) for w in weights])
        h = C.c_void_p()
        plans[0].ctx._check(self._lib.emc_batch_create(hp, hm, hw, n, C.byref(h)), "batch_create")
        self._h = h
        for p in plans:  # the batch goes before any of its plans' contexts
            p.ctx._children.add(self)

    def run(self, sigmas):
        arr = (C.c_float * len(self.plans))(*[float(s) for s in sigmas])
        self.plans[0].ctx._check(self._lib.emc_batch_run(self._h, arr), "batch_run")

    def wait(self):
        st = (IterStats * len(self.plans))()
        self.plans[0].ctx._check(self._lib.emc_batch_wait(self._h, st), "batch_wait")
        return list(st)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.emc_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


for _cls, _names in (
        (Context, ("get_slices", "update_scaling_full", "calculate_responsabilities",
                   "max_vector", "respons_max_expf", "norm_respons_sumexpf", "log_sum_max",
                   "update_slices", "divide_model_by_weight", "normalize_model", "model_max",
                   "model_average", "blur_model", "bin_images", "normalize_images", "mask_model",
                   "model_init_radial", "model_init_orientations", "reset_real", "copy_real_d2d",
                   "copy_real_to_host")),
        (Plan, ("bind", "iterate", "iterate_async", "best_quaternions", "set_proposals",
                "capture", "replay", "autotune", "time_likelihood", "set_pruning", "results",
                "rank_estep", "rank_mstep", "model_from_sums")),
        (Proposal, ("set_data", "loss_grad", "train", "predict"))):
    for _n in _names:
        setattr(_cls, _n, _stream_ordered(getattr(_cls, _n)))
del _cls, _names, _n
