"""C-ABI checks that need no GPU: the library builds and loads, exports every
function include/satgb.h declares, and rejects bad arguments before it
touches the device (the reference has no error reporting at all:
CUDA_CHECK_ERROR is an empty macro, cudaLib.cuh:21-22)."""
import ctypes
import subprocess

import pytest

from sat_gb300 import _lib


def test_exports_every_header_symbol(satlib):
    declared = _lib.header_symbols()
    assert len(declared) >= 23
    out = subprocess.run(["nm", "-D", "--defined-only", _lib._build.lib_path()],
                         capture_output=True, text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = [s for s in declared if s not in exported]
    assert not missing, missing
    for s in declared:
        assert getattr(satlib, s) is not None


def test_version_and_configs(satlib):
    assert satlib.satgb_version() == 100
    n = satlib.satgb_num_configs()
    assert n >= 3
    assert all(satlib.satgb_config_name(i) for i in range(n))
    assert satlib.satgb_config_name(n) == b""


def _call(satlib, fn, in_t, out_t, scan=0, d_in=0x1000, ip=16, d_out=0x100000, op=16, w=16, h=16):
    return getattr(satlib, fn)(in_t, out_t, scan, d_in, ip, d_out, op, w, h, None)


@pytest.mark.parametrize("fn", ["satgb_scanrow_brlt", "satgb_brlt_scanrow", "satgb_scanrowcolumn"])
def test_validation_errors(satlib, fn):
    U8, U32, F32, F64, U16 = _lib.U8, _lib.U32, _lib.F32, _lib.F64, _lib.U16
    assert _call(satlib, fn, U8, U32, w=-1) == _lib.ERR_INVALID_ARG
    assert _call(satlib, fn, U8, U32, h=-5) == _lib.ERR_INVALID_ARG
    assert _call(satlib, fn, U8, U32, scan=2) == _lib.ERR_INVALID_ARG
    assert _call(satlib, fn, U8, U32, d_in=0) == _lib.ERR_INVALID_ARG
    assert _call(satlib, fn, U8, U32, d_out=0) == _lib.ERR_INVALID_ARG
    assert _call(satlib, fn, U8, U32, ip=8) == _lib.ERR_INVALID_ARG          # pitch < width
    assert _call(satlib, fn, U8, U32, op=15) == _lib.ERR_INVALID_ARG
    assert _call(satlib, fn, 9, U32) == _lib.ERR_INVALID_ARG                 # unknown dtype code
    assert _call(satlib, fn, U16, U32) == _lib.ERR_UNSUPPORTED_TYPES        # listed, never dispatched
    assert _call(satlib, fn, F32, U32) == _lib.ERR_UNSUPPORTED_TYPES        # the reference skips f32->u32
    assert _call(satlib, fn, F64, F32) == _lib.ERR_UNSUPPORTED_TYPES
    assert _call(satlib, fn, U8, U32, d_out=0x100002) == _lib.ERR_MISALIGNED
    assert _call(satlib, fn, U8, U32, d_in=0x1000, d_out=0x1008) == _lib.ERR_INVALID_ARG  # overlap
    assert _call(satlib, fn, U8, U32, ip=1 << 62, h=1 << 20) == _lib.ERR_OVERFLOW
    # empty images are a valid no-op and never reach the device
    assert _call(satlib, fn, U8, U32, w=0) == _lib.OK
    assert _call(satlib, fn, U8, U32, h=0, d_in=0, d_out=0) == _lib.OK
    msg = satlib.satgb_last_error_string()
    assert isinstance(msg, bytes)


def test_scan_rows_transposed_validation(satlib):
    """The transposed row scan's output is height wide and width tall: its
    pitch is checked against the height, and the buffers may not overlap."""
    f = satlib.satgb_scan_rows_transposed
    U8, U32 = _lib.U8, _lib.U32

    def call(in_t=U8, out_t=U32, d_in=0x1000, ip=16, d_out=0x100000, op=8, w=16, h=8):
        return f(in_t, out_t, d_in, ip, d_out, op, w, h, None)

    assert call(w=-1) == _lib.ERR_INVALID_ARG
    assert call(d_in=0) == _lib.ERR_INVALID_ARG
    assert call(ip=15) == _lib.ERR_INVALID_ARG               # in pitch < width
    assert call(op=7) == _lib.ERR_INVALID_ARG                # out pitch < height
    assert call(in_t=9) == _lib.ERR_INVALID_ARG
    assert call(in_t=_lib.U16) == _lib.ERR_UNSUPPORTED_TYPES
    assert call(in_t=_lib.F32, out_t=U32) == _lib.ERR_UNSUPPORTED_TYPES
    assert call(d_out=0x100002) == _lib.ERR_MISALIGNED
    assert call(d_out=0x1008) == _lib.ERR_INVALID_ARG        # overlap
    assert call(w=1 << 31, ip=1 << 31) == _lib.ERR_OVERFLOW
    assert call(w=0) == _lib.OK
    assert call(h=0, d_in=0, d_out=0) == _lib.OK


def test_scan_rows_validation(satlib):
    """The row-only scan (its own kernel, no workspace) validates like the
    SAT entry points and offers the same pairs; sizes beyond its kernel's
    32-bit column and row indices are refused before any launch."""
    f = satlib.satgb_scan_rows
    U8, U32 = _lib.U8, _lib.U32

    def call(in_t=U8, out_t=U32, d_in=0x1000, ip=16, d_out=0x10000000000, op=16, w=16, h=8):
        return f(in_t, out_t, d_in, ip, d_out, op, w, h, None)

    assert call(w=-1) == _lib.ERR_INVALID_ARG
    assert call(d_out=0) == _lib.ERR_INVALID_ARG
    assert call(ip=15) == _lib.ERR_INVALID_ARG
    assert call(in_t=_lib.U16) == _lib.ERR_UNSUPPORTED_TYPES
    assert call(in_t=_lib.F32, out_t=U32) == _lib.ERR_UNSUPPORTED_TYPES
    assert call(w=(1 << 31) - 16, ip=1 << 31, op=1 << 31, h=1) == _lib.ERR_OVERFLOW
    assert call(w=0) == _lib.OK
    assert call(h=0, d_in=0, d_out=0) == _lib.OK


def test_box_filter_validation(satlib):
    """Box-filter descriptors are checked before any launch: radii count and
    sign, sizes within the launch grid (height up to 65535 x 32), plane count,
    pitches, alignment; empty sizes are a no-op."""
    def desc(**kw):
        d = _lib.satgb_box_desc()
        d.width, d.height, d.n_planes = kw.get("w", 64), kw.get("h", 64), kw.get("planes", 1)
        d.d_sat, d.sat_pitch, d.sat_plane_stride = kw.get("sat", 0x10000), kw.get("sp", 64), 64 * 64
        d.n_radii = kw.get("n", 1)
        d.radius[0] = kw.get("r", 3)
        d.d_box[0] = kw.get("box", 0x200000)
        d.box_pitch, d.box_plane_stride = kw.get("bp", 64), 64 * 64
        return d

    for fn in (satlib.satgb_box_filter_fwd, satlib.satgb_box_filter_bwd):
        call = lambda **kw: fn(ctypes.byref(desc(**kw)), None)  # noqa: E731
        assert call(n=0) == _lib.ERR_INVALID_ARG
        assert call(n=5) == _lib.ERR_INVALID_ARG
        assert call(r=-1) == _lib.ERR_INVALID_ARG
        assert call(h=65535 * 32 + 1) == _lib.ERR_INVALID_ARG
        assert call(w=(1 << 30) + 1, sp=(1 << 30) + 1, bp=(1 << 30) + 1) == _lib.ERR_INVALID_ARG
        assert call(planes=65536) == _lib.ERR_INVALID_ARG
        assert call(sp=63) == _lib.ERR_INVALID_ARG
        assert call(sat=0) == _lib.ERR_INVALID_ARG
        assert call(box=0) == _lib.ERR_INVALID_ARG
        assert call(sat=0x10002) == _lib.ERR_MISALIGNED
        assert call(box=0x200002) == _lib.ERR_MISALIGNED
        assert call(w=0) == _lib.OK and call(h=0) == _lib.OK and call(planes=0) == _lib.OK


def test_box_grad_x_validation(satlib):
    """satgb_box_filter_bwd_x checks its descriptor like the other box-filter
    calls (the SAT buffer is not needed), then its output: present, aligned,
    pitch and plane stride large enough, no overlap with the gradients read."""
    d = _lib.satgb_box_desc()
    d.width, d.height, d.n_planes = 64, 64, 1
    d.n_radii = 1
    d.radius[0] = 3
    d.d_box[0] = 0x200000
    d.box_pitch, d.box_plane_stride = 64, 64 * 64
    f = satlib.satgb_box_filter_bwd_x
    assert f(ctypes.byref(d), None, 64, 64 * 64, None) == _lib.ERR_INVALID_ARG
    assert f(ctypes.byref(d), 0x300002, 64, 64 * 64, None) == _lib.ERR_MISALIGNED
    assert f(ctypes.byref(d), 0x300000, 63, 64 * 64, None) == _lib.ERR_INVALID_ARG
    assert f(ctypes.byref(d), 0x200000 + 4 * 100, 64, 64 * 64, None) == _lib.ERR_INVALID_ARG  # overlaps g
    d.n_radii = 0
    assert f(ctypes.byref(d), 0x300000, 64, 64 * 64, None) == _lib.ERR_INVALID_ARG
    d.n_radii, d.width = 1, 0
    assert f(ctypes.byref(d), 0x300000, 64, 64 * 64, None) == _lib.OK  # empty: nothing to do


def test_error_string_set_on_failure(satlib):
    assert _call(satlib, "satgb_scanrow_brlt", _lib.U8, _lib.U32, w=-1) == _lib.ERR_INVALID_ARG
    assert b"width" in satlib.satgb_last_error_string()


def test_sat_ex_validation(satlib):
    d = _lib.satgb_sat_desc(_lib.U8, _lib.F32, _lib.MODE_COMPENSATED, _lib.FORWARD, 0x1000, 16, 0x100000, 16, 16, 16)
    # compensated u8 -> f32 is offered; compensated u8 -> u32 is not
    d.out_t = _lib.U32
    assert satlib.satgb_sat_ex(ctypes.byref(d), None) == _lib.ERR_UNSUPPORTED_TYPES
    d.out_t = _lib.F32
    d.direction = 3
    assert satlib.satgb_sat_ex(ctypes.byref(d), None) == _lib.ERR_INVALID_ARG
    d.direction = 0
    d.mode = 7
    assert satlib.satgb_sat_ex(ctypes.byref(d), None) == _lib.ERR_INVALID_ARG
    assert satlib.satgb_sat_ex(None, None) == _lib.ERR_INVALID_ARG


def test_setters_validate(satlib):
    assert satlib.satgb_set_config(99) == _lib.ERR_INVALID_ARG
    assert satlib.satgb_set_config(-1) == _lib.OK
    assert satlib.satgb_set_wait_limit_us(0) == _lib.ERR_INVALID_ARG
    assert satlib.satgb_set_wait_limit_us(2_000_000) == _lib.OK
    assert satlib.satgb_debug_stall_tile(-1) == _lib.OK
    alloc = _lib._ALLOC_FN(lambda n, ctx: None)
    assert satlib.satgb_set_allocator(alloc, _lib._FREE_FN(), None) == _lib.ERR_INVALID_ARG
    assert satlib.satgb_set_allocator(_lib._ALLOC_FN(), _lib._FREE_FN(), None) == _lib.OK


def test_batch_plan_validation(satlib):
    plan = ctypes.c_void_p()
    imgs = (_lib.satgb_image * 1)()
    imgs[0] = _lib.satgb_image(0x1000, 16, 0x100000, 16, -4, 16)
    assert satlib.satgb_batch_plan_create(ctypes.byref(plan), _lib.U8, _lib.U32, 0, 0, imgs, 1, None) == _lib.ERR_INVALID_ARG
    assert satlib.satgb_batch_plan_create(ctypes.byref(plan), _lib.U8, _lib.U32, 0, 0, imgs, 0, None) == _lib.ERR_INVALID_ARG
    assert satlib.satgb_batch_plan_create(None, _lib.U8, _lib.U32, 0, 0, imgs, 1, None) == _lib.ERR_INVALID_ARG
    assert satlib.satgb_batch_plan_exec(None, None) == _lib.ERR_INVALID_ARG
    assert satlib.satgb_batch_plan_destroy(None) == _lib.OK


def test_batch_plan_rejects_images_that_overlap(satlib):
    """The images of a batch run at once, so no image may write memory that
    another image reads or writes; shared inputs and images side by side in
    one pitched buffer are fine.  The check runs before any device call."""
    def create(*images):
        arr = (_lib.satgb_image * len(images))()
        for i, im in enumerate(images):
            arr[i] = _lib.satgb_image(*im)
        plan = ctypes.c_void_p()
        st = satlib.satgb_batch_plan_create(ctypes.byref(plan), _lib.U8, _lib.U32, 0, 0, arr, len(images), None)
        if st == _lib.OK:  # with a GPU: the plan captured its launch but never ran it
            satlib.satgb_batch_plan_destroy(plan)
        return st

    def overlap(st):
        return st == _lib.ERR_INVALID_ARG and b"overlap" in satlib.satgb_last_error_string()

    # (d_in, in_pitch, d_out, out_pitch, width, height); u8 inputs, u32 outputs
    a = (0x100000, 64, 0x800000, 64, 64, 64)
    assert overlap(create(a, (0x200000, 64, 0x800000 + 4 * 64 * 10, 64, 64, 64)))  # outputs overlap
    assert overlap(create(a, (0x800000 + 100, 64, 0x900000, 64, 64, 64)))         # reads image 0's output
    assert overlap(create(a, (0x200000, 64, 0x100000, 16, 16, 16)))               # writes image 0's input
    assert not overlap(create(a, (0x100000, 64, 0x900000, 64, 64, 64)))           # shared input
    # side by side in one pitched buffer (pitch 128 elements): columns 0-63 and 64-127
    b = (0x100000, 128, 0x800000, 128, 64, 64)
    c = (0x100000 + 64, 128, 0x800000 + 4 * 64, 128, 64, 64)
    assert not overlap(create(b, c))
    assert overlap(create(b, (0x100000 + 32, 128, 0x800000 + 4 * 32, 128, 64, 64)))  # columns 32-95


def test_python_api_rejects_cpu_tensors(satlib):
    torch = pytest.importorskip("torch")
    import sat_gb300
    x = torch.zeros(4, 4, dtype=torch.uint8)
    with pytest.raises(sat_gb300.SatError):
        sat_gb300.scanrow_brlt(x, torch.uint32)


def test_cli_usage(satlib):
    """The reference's command line (sat A S D0 D1 R) is built beside the
    library; without arguments it prints its usage and exits 2."""
    import subprocess
    from sat_gb300 import build as B
    r = subprocess.run([B.cli_path()], capture_output=True, text=True)
    assert r.returncode == 2
    assert "sat A S D0 D1 R" in r.stderr
    r = subprocess.run([B.cli_path(), "5", "1", "0", "4", "1"], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr
