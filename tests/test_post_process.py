"""The post-process pass's host side (no GPU): the push-constant layout, the
size-derived defaults of source/taa.hpp:101-111 and 352-359, and the
argument checks of taa_post_process that run before any launch."""
import ctypes as C

import numpy as np
import pytest

import taa_abi as T


def round_half_away(v):
    return np.sign(v) * np.floor(np.abs(v) + np.float32(0.5))


def reference_defaults(w, h):
    """set_source_image_views: w / 96.f etc. in float, std::round, unsigned w."""
    f = lambda d: int(round_half_away(np.float32(w) / np.float32(d)))
    src, dst, brd = f(96.0), f(9.6), f(96.0 * 2.0)
    return (((w - src) // 2, (h - src) // 2, src, src), (w - dst - brd, brd, dst, dst))


def test_params_have_the_push_constant_layout():
    assert C.sizeof(T.PostProcessParams) == 84
    assert T.PostProcessParams.zoom.offset == 64 and T.PostProcessParams.split_x.offset == 72


@pytest.mark.parametrize("size", [(1920, 1080), (3840, 2160), (1280, 720), (72, 48), (1, 1), (333, 17)])
def test_defaults_follow_the_reference(size):
    w, h = size
    p = T.post_process_default_params(w, h)
    src, dst = reference_defaults(w, h)
    assert tuple(p.zoom_src_ltwh) == src and tuple(p.zoom_dst_ltwh) == dst
    assert tuple(p.debug_l_mask) == (1.0, 1.0, 1.0, 0.0) and tuple(p.debug_r_mask) == (1.0, 1.0, 1.0, 0.0)
    assert (p.zoom, p.show_zoom_box, p.split_x, p.debug_l_show, p.debug_r_show) == (0, 1, -1, 0, 0)
    if size == (1920, 1080):  # the struct's own initialisers
        assert src == (950, 530, 20, 20) and dst == (1710, 10, 200, 200)


def test_arguments_are_checked_before_launch():
    lib = T.load()
    p = T.post_process_default_params(64, 32)
    buf = (C.c_uint8 * (64 * 32 * 8 * 3 + 64))()
    base = (C.addressof(buf) + 15) // 16 * 16
    inp, dbg, out = base, base + 64 * 32 * 8, base + 2 * 64 * 32 * 8
    pitch = 64 * 8
    call = lambda params, i, d, o, w=64, h=32, ip=pitch: lib.taa_post_process(
        None, C.byref(params) if params is not None else None, i, ip, d, pitch, o, pitch, w, h)
    assert call(None, inp, dbg, out) == T.TAA_E_INVAL
    assert call(p, inp, dbg, out, w=0) == T.TAA_E_INVAL
    assert call(p, inp, dbg, out, w=32769) == T.TAA_E_INVAL
    assert call(p, None, dbg, out) == T.TAA_E_INVAL
    assert call(p, inp, dbg, inp) == T.TAA_E_INVAL  # output overlaps input
    assert call(p, inp, dbg, out, ip=pitch - 8) == T.TAA_E_INVAL  # pitch below a row
    shown = T.post_process_default_params(64, 32)
    shown.debug_r_show = 1
    assert call(shown, inp, None, out) == T.TAA_E_INVAL  # a side shows the debug image
    assert call(shown, inp, out, out) == T.TAA_E_INVAL  # output overlaps debug
    far = T.post_process_default_params(64, 32)
    far.zoom_dst_ltwh[0] = (1 << 24) + 1
    assert call(far, inp, dbg, out) == T.TAA_E_INVAL
    nan = T.post_process_default_params(64, 32)
    nan.debug_l_mask[3] = float("nan")
    assert call(nan, inp, dbg, out) == T.TAA_E_INVAL
