"""Torch-facing host API over the C ABI.

The reference's operator interface is its three host drivers
``BlockScan::Test``, ``SerielScan::Test`` and ``IncrementScan::Test``
(pengdada/SAT integralImage/ScanRow-BRLT.cu:182-255, BRLT-Scan.cu:192-266,
ScanRowColumn.cu:424-499), each templated over <TSrc, TDst, SCAN_TYPE> and
computing the SAT of a row-major W x H image into a caller-visible device
buffer.  The functions here keep those three names (``scanrow_brlt``,
``brlt_scanrow``, ``scanrowcolumn``), the same type pairs and the same scan
type argument, over torch CUDA tensors (device memory and streams only; the
arithmetic is the CUDA kernel's).

Images are 2-D tensors (height, width) whose rows are contiguous; the row
stride becomes the pitch in elements, as in the reference's GpuData
(cudaLib.cuh:178-180).
"""
from __future__ import annotations

import ctypes
from typing import Optional, Sequence

import torch

from . import _lib
from ._lib import (F32, F64, FORWARD, I8, I32, KOGGE_STONE_SCAN, LF_SCAN, MODE_COMPENSATED,
                   MODE_PLAIN, REVERSE, U8, U32, SatError, check)

_TORCH_TO_CODE = {
    torch.uint8: U8,
    torch.int8: I8,
    torch.uint32: U32,
    torch.int32: I32,
    torch.float32: F32,
    torch.float64: F64,
}
_CODE_TO_TORCH = {v: k for k, v in _TORCH_TO_CODE.items()}

# default output type per input type (the reference's usual pairs)
DEFAULT_OUT = {torch.uint8: torch.uint32, torch.int8: torch.int32, torch.uint32: torch.uint32,
               torch.int32: torch.int32, torch.float32: torch.float32, torch.float64: torch.float64}

# The pairs the reference's host drivers dispatch (ScanRow-BRLT.cu:274-376)
# plus u32 -> u32.
PAIRS = [
    (torch.uint8, torch.uint32), (torch.uint8, torch.float32), (torch.uint8, torch.float64),
    (torch.int8, torch.int32), (torch.int8, torch.float32), (torch.int8, torch.float64),
    (torch.int32, torch.int32), (torch.int32, torch.float64),
    (torch.uint32, torch.uint32),
    (torch.float32, torch.float32), (torch.float32, torch.float64),
    (torch.float64, torch.float64),
]

_MODES = {"plain": MODE_PLAIN, "compensated": MODE_COMPENSATED}


def dtype_code(dt: torch.dtype) -> int:
    try:
        return _TORCH_TO_CODE[dt]
    except KeyError:
        raise SatError(_lib.ERR_UNSUPPORTED_TYPES, f"dtype {dt} has no satgb_dtype code") from None


def _stream_handle(stream) -> int:
    if stream is None:
        stream = torch.cuda.current_stream()
    return int(stream.cuda_stream) if hasattr(stream, "cuda_stream") else int(stream)


def _image_args(t: torch.Tensor):
    if t.dim() != 2:
        raise SatError(_lib.ERR_INVALID_ARG, f"an image is a 2-D tensor, got shape {tuple(t.shape)}")
    h, w = t.shape
    if w > 1 and t.stride(1) != 1:
        raise SatError(_lib.ERR_INVALID_ARG, "image rows must be contiguous (stride(1) == 1)")
    pitch = t.stride(0) if h > 1 else max(w, t.stride(0))
    return t.data_ptr(), int(pitch), int(w), int(h)


def _check_cuda(*ts: torch.Tensor) -> None:
    for t in ts:
        if not t.is_cuda:
            raise SatError(_lib.ERR_INVALID_ARG, "tensors must be CUDA tensors (there is no CPU path)")


def _prep_out(src: torch.Tensor, out_dtype, out: Optional[torch.Tensor]) -> torch.Tensor:
    if out_dtype is None:
        out_dtype = out.dtype if out is not None else DEFAULT_OUT.get(src.dtype, src.dtype)
    if out is None:
        out = torch.empty(src.shape, dtype=out_dtype, device=src.device)
    elif out.dtype != out_dtype or out.shape != src.shape:
        raise SatError(_lib.ERR_INVALID_ARG, "out has the wrong dtype or shape")
    return out


def _three(fn_name: str, src: torch.Tensor, out_dtype, scan_type: int, out, stream) -> torch.Tensor:
    _check_cuda(src)
    out = _prep_out(src, out_dtype, out)
    _check_cuda(out)
    ip, ipitch, w, h = _image_args(src)
    op, opitch, _, _ = _image_args(out)
    L = _lib.load()
    check(getattr(L, fn_name)(dtype_code(src.dtype), dtype_code(out.dtype), int(scan_type), ip, ipitch,
                              op, opitch, w, h, _stream_handle(stream)))
    return out


def scanrow_brlt(src: torch.Tensor, out_dtype=None, scan_type: int = LF_SCAN, out=None, stream=None):
    """ScanRow-BRLT (BlockScan): SAT of `src` (BlockScan::Test, ScanRow-BRLT.cu:182-255)."""
    return _three("satgb_scanrow_brlt", src, out_dtype, scan_type, out, stream)


def brlt_scanrow(src: torch.Tensor, out_dtype=None, scan_type: int = LF_SCAN, out=None, stream=None):
    """BRLT-ScanRow (SerialScan): SAT of `src` (SerielScan::Test, BRLT-Scan.cu:192-266)."""
    return _three("satgb_brlt_scanrow", src, out_dtype, scan_type, out, stream)


def scanrowcolumn(src: torch.Tensor, out_dtype=None, scan_type: int = LF_SCAN, out=None, stream=None):
    """ScanRowColumn (IncreamentScan): SAT of `src` (IncrementScan::Test, ScanRowColumn.cu:424-499)."""
    return _three("satgb_scanrowcolumn", src, out_dtype, scan_type, out, stream)


def _scan(fn_name: str, src: torch.Tensor, out_dtype, out, stream) -> torch.Tensor:
    _check_cuda(src)
    out = _prep_out(src, out_dtype, out)
    _check_cuda(out)
    ip, ipitch, w, h = _image_args(src)
    op, opitch, _, _ = _image_args(out)
    check(getattr(_lib.load(), fn_name)(dtype_code(src.dtype), dtype_code(out.dtype), ip, ipitch, op, opitch, w, h,
                                        _stream_handle(stream)))
    return out


def scan_rows(src: torch.Tensor, out_dtype=None, out=None, stream=None) -> torch.Tensor:
    """Row-only scan, out(y,x) = sum_{i<=x} src(y,i) (IncrementScanX, IncrementScanX.cu:12-113)."""
    return _scan("satgb_scan_rows", src, out_dtype, out, stream)


def scan_cols(src: torch.Tensor, out_dtype=None, out=None, stream=None) -> torch.Tensor:
    """Column-only scan, out(y,x) = sum_{j<=y} src(j,x) (IncrementScanY, IncrementScanY.cu:10-126)."""
    return _scan("satgb_scan_cols", src, out_dtype, out, stream)


def scan_rows_transposed(src: torch.Tensor, out_dtype=None, out=None, stream=None) -> torch.Tensor:
    """Row scan with transposed output, out(x, y) = sum_{i<=x} src(y, i): an
    (H, W) input gives a (W, H) output (SerielScan::TestX, BRLT-Scan.cu:128-190)."""
    _check_cuda(src)
    if src.dim() != 2:
        raise SatError(_lib.ERR_INVALID_ARG, f"an image is a 2-D tensor, got shape {tuple(src.shape)}")
    if out_dtype is None:
        out_dtype = out.dtype if out is not None else DEFAULT_OUT.get(src.dtype, src.dtype)
    shape_t = (src.shape[1], src.shape[0])
    if out is None:
        out = torch.empty(shape_t, dtype=out_dtype, device=src.device)
    elif out.dtype != out_dtype or tuple(out.shape) != shape_t:
        raise SatError(_lib.ERR_INVALID_ARG, "out has the wrong dtype or shape (it is the transposed shape)")
    _check_cuda(out)
    ip, ipitch, w, h = _image_args(src)
    op, opitch, _, _ = _image_args(out)
    check(_lib.load().satgb_scan_rows_transposed(dtype_code(src.dtype), dtype_code(out.dtype), ip, ipitch, op, opitch,
                                                 w, h, _stream_handle(stream)))
    return out


ALGORITHMS = {
    "ScanRow-BRLT": scanrow_brlt,
    "BRLT-ScanRow": brlt_scanrow,
    "ScanRowColumn": scanrowcolumn,
}


def _planes_args(t: torch.Tensor):
    """(ptr, pitch, width, height, n_planes, plane_stride) of a (..., H, W)
    tensor whose leading dimensions collapse into one plane stride."""
    if t.dim() < 3:
        raise SatError(_lib.ERR_INVALID_ARG, f"expected a (..., H, W) tensor, got shape {tuple(t.shape)}")
    h, w = t.shape[-2], t.shape[-1]
    try:
        v = t.view(-1, h, w)
    except RuntimeError:
        raise SatError(_lib.ERR_INVALID_ARG, "leading dimensions must collapse into one plane stride") from None
    if w > 1 and v.stride(2) != 1:
        raise SatError(_lib.ERR_INVALID_ARG, "image rows must be contiguous (stride(-1) == 1)")
    pitch = v.stride(1) if h > 1 else max(w, v.stride(1))
    n = v.shape[0]
    plane = v.stride(0) if n > 1 else pitch * h
    return v.data_ptr(), int(pitch), int(w), int(h), int(n), int(plane)


def sat(src: torch.Tensor, out_dtype=None, mode: str = "plain", reverse: bool = False, out=None,
        stream=None) -> torch.Tensor:
    """SAT (or, with reverse=True, the suffix SAT) of a 2-D image, or of every
    (H, W) plane of a (..., H, W) tensor in one launch; mode "compensated"
    carries two-sum error terms (f32 outputs)."""
    _check_cuda(src)
    out = _prep_out(src, out_dtype, out)
    _check_cuda(out)
    direction = REVERSE if reverse else FORWARD
    if src.dim() >= 3:
        ip, ipitch, w, h, n, iplane = _planes_args(src)
        op, opitch, _, _, _, oplane = _planes_args(out)
        d = _lib.satgb_sat_desc(dtype_code(src.dtype), dtype_code(out.dtype), _MODES[mode], direction,
                                ip, ipitch, op, opitch, w, h)
        check(_lib.load().satgb_sat_planes(ctypes.byref(d), n, iplane, oplane, _stream_handle(stream)))
        return out
    ip, ipitch, w, h = _image_args(src)
    op, opitch, _, _ = _image_args(out)
    d = _lib.satgb_sat_desc(dtype_code(src.dtype), dtype_code(out.dtype), _MODES[mode], direction,
                            ip, ipitch, op, opitch, w, h)
    check(_lib.load().satgb_sat_ex(ctypes.byref(d), _stream_handle(stream)))
    return out


def _box_desc(sat_t: torch.Tensor, boxes: torch.Tensor, radii: Sequence[int]):
    """satgb_box_desc for a (..., H, W) f32 SAT and a (..., R, H, W) f32 box
    tensor (one (H, W) plane per radius)."""
    if sat_t.dtype != torch.float32 or boxes.dtype != torch.float32:
        raise SatError(_lib.ERR_UNSUPPORTED_TYPES, "box filters take f32 tensors")
    radii = [int(r) for r in radii]
    if not 1 <= len(radii) <= _lib.MAX_RADII or min(radii) < 0:
        raise SatError(_lib.ERR_INVALID_ARG, f"1..{_lib.MAX_RADII} non-negative radii, got {radii}")
    if boxes.shape != sat_t.shape[:-2] + (len(radii),) + sat_t.shape[-2:]:
        raise SatError(_lib.ERR_INVALID_ARG, "box tensor must be (..., R, H, W)")
    _check_cuda(sat_t, boxes)
    s3 = sat_t if sat_t.dim() >= 3 else sat_t.unsqueeze(0)
    sp, spitch, w, h, n, splane = _planes_args(s3)
    b4 = boxes.reshape((-1, len(radii)) + boxes.shape[-2:]) if boxes.dim() >= 4 else boxes.unsqueeze(0)
    if b4.data_ptr() != boxes.data_ptr() or b4.stride(-1) != 1:
        raise SatError(_lib.ERR_INVALID_ARG, "box tensor must be contiguous in its last dimension")
    d = _lib.satgb_box_desc()
    d.width, d.height, d.n_planes = w, h, n
    d.d_sat, d.sat_pitch, d.sat_plane_stride = sp, spitch, splane
    d.n_radii = len(radii)
    esz = boxes.element_size()
    for i, r in enumerate(radii):
        d.radius[i] = r
        d.d_box[i] = b4.data_ptr() + i * b4.stride(1) * esz
    d.box_pitch = b4.stride(2) if h > 1 else max(w, b4.stride(2))
    d.box_plane_stride = b4.stride(0) if n > 1 else d.box_pitch * h
    return d


def box_means_from_sat(sat_t: torch.Tensor, radii: Sequence[int], out=None, stream=None) -> torch.Tensor:
    """Clipped box means of every radius from an f32 SAT: (..., H, W) ->
    (..., R, H, W)."""
    if out is None:
        out = torch.empty(sat_t.shape[:-2] + (len(radii),) + sat_t.shape[-2:], dtype=torch.float32,
                          device=sat_t.device)
    d = _box_desc(sat_t, out, radii)
    check(_lib.load().satgb_box_filter_fwd(ctypes.byref(d), _stream_handle(stream)))
    return out


def box_means_adjoint(grad_boxes: torch.Tensor, radii: Sequence[int], out=None, stream=None) -> torch.Tensor:
    """The adjoint of box_means_from_sat: dL/dSAT (..., H, W) from dL/dmeans
    (..., R, H, W)."""
    if out is None:
        out = torch.empty(grad_boxes.shape[:-3] + grad_boxes.shape[-2:], dtype=torch.float32,
                          device=grad_boxes.device)
    d = _box_desc(out, grad_boxes, radii)
    check(_lib.load().satgb_box_filter_bwd(ctypes.byref(d), _stream_handle(stream)))
    return out


def box_means_grad_x(grad_boxes: torch.Tensor, radii: Sequence[int], out=None, stream=None) -> torch.Tensor:
    """dL/dx of the box means of x from dL/dmeans (..., R, H, W) in one call:
    the adjoint gather writes dL/dSAT into out, which is then reverse-summed
    in place (no scratch tensor)."""
    shape = grad_boxes.shape[:-3] + grad_boxes.shape[-2:]
    if out is None:
        out = torch.empty(shape, dtype=torch.float32, device=grad_boxes.device)
    elif out.shape != shape or out.dtype != torch.float32:
        raise SatError(_lib.ERR_INVALID_ARG, "out must be an f32 (..., H, W) tensor")
    d = _box_desc(out, grad_boxes, radii)
    o3 = out if out.dim() >= 3 else out.unsqueeze(0)
    _, opitch, _, _, _, oplane = _planes_args(o3)
    d.d_sat = None
    check(_lib.load().satgb_box_filter_bwd_x(ctypes.byref(d), out.data_ptr(), opitch, oplane, _stream_handle(stream)))
    return out


def stream_check(stream=None) -> None:
    """Synchronises the stream and raises SatError(SATGB_ERR_TIMEOUT) when a
    look-back wait of an earlier call gave up."""
    check(_lib.load().satgb_stream_check(_stream_handle(stream)))


def autotune(src: torch.Tensor, out: torch.Tensor, mode: str = "plain", stream=None) -> int:
    """Times every tile configuration on (src, out) and records the best."""
    _check_cuda(src, out)
    ip, ipitch, w, h = _image_args(src)
    op, opitch, _, _ = _image_args(out)
    best = ctypes.c_int(-1)
    check(_lib.load().satgb_autotune(dtype_code(src.dtype), dtype_code(out.dtype), _MODES[mode], ip, ipitch,
                                     op, opitch, w, h, _stream_handle(stream), ctypes.byref(best)))
    return best.value


def set_config(config: int) -> None:
    check(_lib.load().satgb_set_config(int(config)))


def config_names() -> list:
    L = _lib.load()
    return [L.satgb_config_name(i).decode() for i in range(L.satgb_num_configs())]


def set_wait_limit_us(us: int) -> None:
    check(_lib.load().satgb_set_wait_limit_us(int(us)))


def release() -> None:
    check(_lib.load().satgb_release())


class BatchPlan:
    """Many images of uneven sizes in one persistent launch captured in a CUDA
    graph (satgb_batch_plan_*).  The tensors must stay alive while the plan is
    used; ``exec()`` replays the graph, ``launch()`` launches directly."""

    def __init__(self, inputs: Sequence[torch.Tensor], outputs: Sequence[torch.Tensor],
                 mode: str = "plain", reverse: bool = False, stream=None):
        if len(inputs) != len(outputs) or not inputs:
            raise SatError(_lib.ERR_INVALID_ARG, "inputs and outputs must be equal-length, non-empty lists")
        in_dt, out_dt = inputs[0].dtype, outputs[0].dtype
        arr = (_lib.satgb_image * len(inputs))()
        for i, (a, b) in enumerate(zip(inputs, outputs)):
            _check_cuda(a, b)
            if a.dtype != in_dt or b.dtype != out_dt or a.shape != b.shape:
                raise SatError(_lib.ERR_INVALID_ARG, f"image {i}: mixed dtypes or shape mismatch")
            ip, ipitch, w, h = _image_args(a)
            op, opitch, _, _ = _image_args(b)
            arr[i] = _lib.satgb_image(ip, ipitch, op, opitch, w, h)
        self._keep = (list(inputs), list(outputs))
        self._plan = ctypes.c_void_p()
        check(_lib.load().satgb_batch_plan_create(ctypes.byref(self._plan), dtype_code(in_dt), dtype_code(out_dt),
                                                  _MODES[mode], REVERSE if reverse else FORWARD, arr,
                                                  len(inputs), _stream_handle(stream)))

    def exec(self, stream=None) -> None:
        check(_lib.load().satgb_batch_plan_exec(self._plan, _stream_handle(stream)))

    def launch(self, stream=None) -> None:
        check(_lib.load().satgb_batch_plan_launch(self._plan, _stream_handle(stream)))

    def check(self, stream=None) -> None:
        check(_lib.load().satgb_batch_plan_check(self._plan, _stream_handle(stream)))

    def info(self):
        n = ctypes.c_int64()
        c = ctypes.c_int()
        check(_lib.load().satgb_batch_plan_info(self._plan, ctypes.byref(n), ctypes.byref(c)))
        return {"n_tiles": n.value, "config": c.value}

    def classes(self):
        """Per size class (large, small): image count, tiles and configuration."""
        n = (ctypes.c_int64 * 2)()
        t = (ctypes.c_int64 * 2)()
        c = (ctypes.c_int * 2)()
        check(_lib.load().satgb_batch_plan_classes(self._plan, n, t, c))
        return [{"images": n[i], "tiles": t[i], "config": c[i]} for i in range(2)]

    def autotune(self, stream=None):
        """Times every tile configuration per size class on this plan's images
        (overwriting the outputs), keeps the fastest and records it in the
        tuning cache; returns the chosen configurations (large, small)."""
        c = (ctypes.c_int * 2)()
        check(_lib.load().satgb_batch_plan_autotune(self._plan, _stream_handle(stream), c))
        return (c[0], c[1])

    def close(self) -> None:
        if self._plan:
            _lib.load().satgb_batch_plan_destroy(self._plan)
            self._plan = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
