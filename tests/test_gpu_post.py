"""The post-process pass (shaders/post_process.comp) on the GPU, run with -m
gpu: the kernel behind taa_post_process gives the FP32 oracle's values after
the RGBA16F store, bit for bit - on the golden fixture's seven push-constant
cases (the oracle there equals the reference shader), at ragged sizes with
padded pitches, split lines at and beyond the edges, zoom boxes partly outside
the image (the fetch clamps) and masks that show or hide the debug alpha, and
at 4K with the size-derived defaults."""
import json
from pathlib import Path

import numpy as np
import pytest
import torch

import oracle as O
import taa_abi as T

pytestmark = pytest.mark.gpu

POST = np.load(Path(__file__).parent / "golden" / "post_golden.npz")


def params_of(pp):
    p = T.PostProcessParams()
    for i in range(4):
        p.zoom_src_ltwh[i] = int(pp["zoom_src"][i])
        p.zoom_dst_ltwh[i] = int(pp["zoom_dst"][i])
        p.debug_l_mask[i] = float(pp["mask_l"][i])
        p.debug_r_mask[i] = float(pp["mask_r"][i])
    p.zoom, p.show_zoom_box = int(bool(pp["zoom"])), int(bool(pp["show_zoom_box"]))
    p.split_x, p.debug_l_show, p.debug_r_show = int(pp["split_x"]), int(bool(pp["show_l"])), int(bool(pp["show_r"]))
    return p


def padded(a16, dev, pad):
    h, w = a16.shape[:2]
    t = torch.zeros(h, w + pad, 4, dtype=torch.float16, device=dev)
    t[:, :w] = torch.from_numpy(a16).to(dev)
    return t[:, :w]


def run(dev, img, dbg, pp, pad=0, with_debug=True):
    src = padded(img.astype(np.float16), dev, pad)
    d = padded(dbg.astype(np.float16), dev, pad + 3) if with_debug else None
    out = torch.full((img.shape[0], img.shape[1] + pad + 1, 4), float("nan"), dtype=torch.float16, device=dev)
    out = out[:, :img.shape[1]]
    T.post_process(src, out, params_of(pp), debug=d)
    torch.cuda.synchronize()
    return out.float().cpu().numpy()


def expected(img, dbg, pp):
    r = O.post_process(img, dbg, precision=32, **{k: v for k, v in pp.items()})
    return r.astype(np.float32).astype(np.float16).astype(np.float32)


def golden_params(name):
    pp = json.loads(str(POST[f"{name}/params"]))
    return {k: tuple(v) if isinstance(v, list) else v for k, v in pp.items()}


@pytest.mark.parametrize("name", sorted({k.split("/")[0] for k in POST.files if "/" in k}))
def test_golden_cases(cuda, name):
    pp = golden_params(name)
    got = run(cuda, POST["image"], POST["debug"], pp)
    ref = POST[f"{name}/ref32"].astype(np.float16).astype(np.float32)
    np.testing.assert_array_equal(got, ref)


RAGGED = {
    "split_at_0": dict(split_x=0, show_r=True, mask_r=(1, 1, 1, 1)),
    "split_at_last_column": dict(split_x=96, show_l=True),
    "split_beyond": dict(split_x=200, show_r=True),
    "negative_split_shows_left": dict(split_x=-7, show_l=True, mask_l=(0, 0, 0, -1)),
    "zoom_source_leaves_the_image": dict(zoom=True, zoom_src=(88, -4, 20, 12), zoom_dst=(5, 30, 33, 29)),
    "zoom_inset_leaves_the_image": dict(zoom=True, zoom_src=(10, 10, 5, 5), zoom_dst=(80, 50, 40, 40),
                                        show_r=True, split_x=60),
    "zoom_degenerate_boxes": dict(zoom=True, zoom_src=(30, 20, 0, 0), zoom_dst=(40, 10, 1, 1)),
    "zoom_hidden_box": dict(zoom=True, show_zoom_box=False, zoom_src=(0, 0, 97, 61), zoom_dst=(0, 0, 97, 61)),
}


@pytest.mark.parametrize("name", list(RAGGED))
def test_ragged_cases(cuda, name):
    rng = np.random.default_rng(len(name))
    h, w = 61, 97
    img = rng.uniform(-2.0, 30.0, (h, w, 4)).astype(np.float16).astype(np.float32)
    dbg = rng.uniform(-1.0, 1.0, (h, w, 4)).astype(np.float16).astype(np.float32)
    pp = dict(O.POST_DEFAULTS)
    pp.update(RAGGED[name])
    shows = pp["show_l"] or pp["show_r"]
    got = run(cuda, img, dbg, pp, pad=5, with_debug=shows)
    np.testing.assert_array_equal(got, expected(img, dbg if shows else None, pp))


def test_4k_size_defaults(cuda):
    w, h = 3840, 2160
    rng = np.random.default_rng(3)
    img = rng.uniform(0.0, 8.0, (h, w, 4)).astype(np.float16).astype(np.float32)
    dbg = rng.uniform(0.0, 1.0, (h, w, 4)).astype(np.float16).astype(np.float32)
    p = T.post_process_default_params(w, h)
    pp = dict(zoom_src=tuple(p.zoom_src_ltwh), zoom_dst=tuple(p.zoom_dst_ltwh), mask_l=(1, 1, 1, 1),
              mask_r=tuple(p.debug_r_mask), zoom=True, show_zoom_box=True, split_x=w // 2, show_l=True, show_r=False)
    got = run(cuda, img, dbg, pp)
    np.testing.assert_array_equal(got, expected(img, dbg, pp))
