"""The tensor-core weight images' layout (csrc/nrc.h, nrc_tc_param_offsets),
checked on the host: the training step's Adam kernel writes every parameter
straight into these images, so each parameter must land on its own bf16
slot, at the (row, K) position the MMA operand layout gives it, and the
padding must stay untouched. A small C++ program compiled against the
header decodes every offset independently of the encoder.
"""
from __future__ import annotations

import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "aqua-engine_gb300", "csrc")

PROGRAM = r"""
#include "nrc.h"
#include <cstdio>
#include <vector>

using namespace aq;

// (row, k) of a byte offset in an R-row tile: core matrices of 8 rows x 16 B,
// one 8-column K slice after another.
static void decode(uint32_t off, int rows, int& r, int& k) {
    const uint32_t slice = (uint32_t)rows * 16;
    r = (int)((off % slice) / 16);
    k = (int)((off / slice) * 8 + (off % 16) / 2);
}

int main() {
    const int hidden = kNrcHiddenLayers * kNrcHidden * kNrcIn;
    const uint32_t fwd_bytes = 5 * kNrcTcLayerBytes + kNrcTcOutRows * 64 * 2;
    const uint32_t bwd_bytes = kNrcTcBwdW6Bytes + 4 * kNrcTcLayerBytes;
    std::vector<int> fwd_used(fwd_bytes / 2, -1), bwd_used(bwd_bytes / 2, -1);
    int errors = 0;
    for (int p = 0; p < kNrcParams; ++p) {
        uint32_t f;
        int32_t b;
        nrc_tc_param_offsets(p, f, b);
        const bool out_layer = p >= hidden;
        const int l = out_layer ? 5 : p / 4096;
        const int o = out_layer ? (p - hidden) / 64 : (p / 64) % 64, i = p % 64;
        if (f % 2 || f >= fwd_bytes || fwd_used[f / 2] >= 0) { printf("fwd slot %d\n", p); ++errors; continue; }
        fwd_used[f / 2] = p;
        int r, k;
        const uint32_t base = (uint32_t)l * kNrcTcLayerBytes;
        decode(f - base, out_layer ? kNrcTcOutRows : 64, r, k);
        if (f < base || r != o || k != i) { printf("fwd place %d\n", p); ++errors; }
        if (l == 0) {
            if (b != -1) { printf("W1 in bwd %d\n", p); ++errors; }
            continue;
        }
        if (b < 0 || b % 2 || (uint32_t)b >= bwd_bytes || bwd_used[b / 2] >= 0) { printf("bwd slot %d\n", p); ++errors; continue; }
        bwd_used[b / 2] = p;
        // backward image: W6^T first (64 rows = inputs, K = 16 outputs), then W5^T..W2^T
        const uint32_t bbase = out_layer ? 0u : (uint32_t)(kNrcTcBwdW6Bytes + (4 - l) * kNrcTcLayerBytes);
        decode((uint32_t)b - bbase, 64, r, k);
        if ((uint32_t)b < bbase || r != i || k != o) { printf("bwd place %d\n", p); ++errors; }
    }
    // every hidden-layer slot is a parameter; the output tiles hold 3 of 16 rows / K columns
    int fwd_free = 0, bwd_free = 0;
    for (int v : fwd_used) fwd_free += v < 0;
    for (int v : bwd_used) bwd_free += v < 0;
    if (fwd_free != (kNrcTcOutRows - kNrcOut) * 64) { printf("fwd padding %d\n", fwd_free); ++errors; }
    if (bwd_free != (16 - kNrcOut) * 64) { printf("bwd padding %d\n", bwd_free); ++errors; }
    printf(errors ? "FAIL %d\n" : "OK\n", errors);
    return errors ? 1 : 0;
}
"""


def test_weight_image_layout(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no host C++ compiler")
    src = tmp_path / "layout.cpp"
    exe = tmp_path / "layout"
    src.write_text(PROGRAM)
    subprocess.run([gxx, "-std=c++17", "-O1", "-I", CSRC, str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0 and out.stdout.strip().endswith("OK"), out.stdout
