"""Writes tests/golden/jpeg_facts.json: the reference scene's JPEG textures
(scenes/textures/*.jpg) decoded by nvJPEG (the CUDA toolkit's decoder) and by
libaqua's own decoder, compared pixel by pixel.

Run on a machine with a GPU and the CUDA toolkit, with the texture directory
as the first argument:

    python tests/golden/make_jpeg_facts.py <dir with the .jpg files> [out.json]

Per file it records the size, the frame type, nvJPEG's mean RGB, and the
mean / maximum absolute difference between the two decoders (both round to
8 bits, so IDCT and chroma-upsampling choices show up as small differences).
The CPU test compares libaqua's mean RGB with nvJPEG's.
"""
from __future__ import annotations

import ctypes as C
import glob
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "aqua-engine_gb300"))


def load_nvjpeg():
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    for d in (os.path.join(cuda, "lib64"), *glob.glob(os.path.join(cuda, "targets", "*", "lib"))):
        for name in ("libnvjpeg.so.13", "libnvjpeg.so"):
            p = os.path.join(d, name)
            if os.path.exists(p):
                return C.CDLL(p)
    raise OSError("libnvjpeg not found")


class NvImage(C.Structure):
    _fields_ = [("channel", C.c_void_p * 4), ("pitch", C.c_size_t * 4)]


NVJPEG_OUTPUT_RGBI = 5


def nvjpeg_decode(lib, handle, state, data: bytes):
    import torch

    nc = C.c_int()
    css = C.c_int()
    ws = (C.c_int * 4)()
    hs = (C.c_int * 4)()
    st = lib.nvjpegGetImageInfo(handle, data, len(data), C.byref(nc), C.byref(css), ws, hs)
    assert st == 0, st
    w, h = ws[0], hs[0]
    buf = torch.zeros(h * w * 3, dtype=torch.uint8, device="cuda")
    img = NvImage()
    img.channel[0] = buf.data_ptr()
    img.pitch[0] = w * 3
    st = lib.nvjpegDecode(handle, state, data, len(data), NVJPEG_OUTPUT_RGBI, C.byref(img),
                          C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0, st
    torch.cuda.synchronize()
    return buf.cpu().numpy().reshape(h, w, 3)


def frame_type(data: bytes) -> str:
    i = 2
    while i + 4 <= len(data):
        m = data[i + 1]
        if m in (0xC0, 0xC1):
            return "sequential"
        if m == 0xC2:
            return "progressive"
        i += 2 + ((data[i + 2] << 8) | data[i + 3])
    return "unknown"


def main():
    import aqua

    src = sys.argv[1]
    out = sys.argv[2] if len(sys.argv) > 2 else os.path.join(HERE, "jpeg_facts.json")
    lib = load_nvjpeg()
    P = C.c_void_p
    lib.nvjpegCreateSimple.argtypes = [C.POINTER(P)]
    lib.nvjpegJpegStateCreate.argtypes = [P, C.POINTER(P)]
    lib.nvjpegGetImageInfo.argtypes = [P, C.c_char_p, C.c_size_t, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                       C.POINTER(C.c_int), C.POINTER(C.c_int)]
    lib.nvjpegDecode.argtypes = [P, P, C.c_char_p, C.c_size_t, C.c_int, C.POINTER(NvImage), P]
    lib.nvjpegJpegStateDestroy.argtypes = [P]
    lib.nvjpegDestroy.argtypes = [P]
    handle, state = C.c_void_p(), C.c_void_p()
    assert lib.nvjpegCreateSimple(C.byref(handle)) == 0
    assert lib.nvjpegJpegStateCreate(handle, C.byref(state)) == 0
    ctx = aqua.Context(device=0)
    facts = {}
    for path in sorted(glob.glob(os.path.join(src, "*.jpg"))):
        data = open(path, "rb").read()
        ref = nvjpeg_decode(lib, handle, state, data).astype(np.int16)
        ours = ctx.decode_jpeg(data).astype(np.int16)
        assert ours.shape == ref.shape, (path, ours.shape, ref.shape)
        d = np.abs(ours - ref)
        facts[os.path.basename(path)] = {
            "width": int(ref.shape[1]), "height": int(ref.shape[0]), "frame": frame_type(data),
            "nvjpeg_mean_rgb": [round(float(x), 4) for x in ref.reshape(-1, 3).mean(0)],
            "mean_abs_diff": round(float(d.mean()), 5), "max_abs_diff": int(d.max()),
            "frac_diff_gt_2": round(float((d > 2).mean()), 6),
        }
        print(os.path.basename(path), facts[os.path.basename(path)], flush=True)
    lib.nvjpegJpegStateDestroy(state)
    lib.nvjpegDestroy(handle)
    with open(out, "w") as f:
        json.dump({"decoder": "nvJPEG (CUDA toolkit), NVJPEG_OUTPUT_RGBI", "files": facts}, f, indent=1,
                  sort_keys=True)


if __name__ == "__main__":
    main()
