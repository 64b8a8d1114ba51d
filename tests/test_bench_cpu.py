"""bench.py's roofline accounting on the CPU: the algorithmic bytes of each
step kernel (its share of the compulsory bytes of a fused step: N*[ns*32 + the
B(k) table]), the bytes each kernel of the 4-pass design moves, the stored B(k)
at 128^3 x 12, computed by hand from the data layout, and the committed ncu
DRAM traffic against the kernel bytes (no kernel re-reads)."""
import json
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]

N = 128 ** 3
NS = 12
P = NS * (NS + 1) // 2  # packed symmetric pairs
INNER = 128 * 128       # x lines per field
TILES = 8320            # mirrored tile table of 128^3: 8064 line pairs + 256 single lines


@pytest.fixture(scope="module")
def bench():
    import bench as b
    return b


def test_b_table_bytes(bench):
    # FP64: every point, 8 bytes a pair
    assert bench.b_table_bytes("fp64", (128, 128, 128), NS) == P * N * 8
    # FP32 mirrored table: a pair row of N1 + 4 values, a single line N1 values
    pairs, singles = INNER - TILES, 2 * TILES - INNER
    assert (pairs, singles) == (8064, 256)
    b = bench.b_table_bytes("fp32", (128, 128, 128), NS, {"x_pass": {"b_tiles": TILES}})
    assert b == P * (pairs * 132 + singles * 128) * 4 == 342331392
    # no table reported: the full FP32 table; closed form: none
    assert bench.b_table_bytes("fp32", (128, 128, 128), NS) == P * N * 4
    assert bench.b_table_bytes("fp32_bfly", (128, 128, 128), NS) == 0


def test_algorithmic_bytes_per_kernel(bench):
    b = 342331392
    # the step's compulsory bytes: xi (complex128) in and out, owned by the z-pass,
    # and one read of the stored B(k), owned by the x-pass; the y passes own none
    assert bench.algorithmic_bytes("z_step", "fp32", N, NS, NS) == NS * N * 32 == 805306368
    assert bench.algorithmic_bytes("x_fused", "fp32", N, NS, NS, b) == b
    assert bench.algorithmic_bytes("fft_y_fwd", "fp32", N, NS, NS) == 0
    assert bench.algorithmic_bytes("z_step", "fp64", N, NS, NS) == NS * N * 32
    total = sum(bench.algorithmic_bytes(k, "fp32", N, NS, NS, b) for k in ("z_step", "x_fused", "fft_y_fwd",
                                                                           "fft_y_inv"))
    assert total == N * (NS * 32) + b


def test_kernel_bytes_per_kernel(bench):
    # z-pass: S (complex64) in and out + FP64 xi (16 bytes) in and out
    assert bench.kernel_bytes("z_step", "fp32", N, NS, NS) == NS * N * (8 + 8 + 16 + 16) == 1207959552
    # y FFT: S in and out
    assert bench.kernel_bytes("fft_y_fwd", "fp32", N, NS, NS) == NS * N * 16
    # x-pass: S in and out + the B table
    b = 342331392
    assert bench.kernel_bytes("x_fused", "fp32", N, NS, NS, b) == NS * N * 16 + b == 744984576
    # FP64 spectra: 16-byte elements
    assert bench.kernel_bytes("z_step", "fp64", N, NS, NS) == NS * N * (16 + 16 + 16 + 16)


def test_committed_traffic_within_algorithmic_bytes(bench):
    traffic = json.loads((ROOT / "profiles" / "traffic.json").read_text())
    b = bench.b_table_bytes("fp32", (128, 128, 128), NS, {"x_pass": {"b_tiles": TILES}})
    expect = {
        "z_step/fp32/128^3x12": bench.kernel_bytes("z_step", "fp32", N, NS, NS),
        "fft_y_fwd/fp32/128^3x12": bench.kernel_bytes("fft_y_fwd", "fp32", N, NS, NS),
        "fft_y_inv/fp32/128^3x12": bench.kernel_bytes("fft_y_inv", "fp32", N, NS, NS),
        "x_fused/fp32/128^3x12": bench.kernel_bytes("x_fused", "fp32", N, NS, NS, b),
        "x_fused/fp32_bfly/128^3x12": bench.kernel_bytes("x_fused", "fp32_bfly", N, NS, NS),
    }
    assert set(expect) <= set(traffic)
    for k, alg in expect.items():
        # DRAM reads + writes of one launch: at most the kernel's bytes
        # (writes come out lower when the last tiles are still in L2 at the end)
        assert 0.8 * alg <= traffic[k] <= 1.01 * alg, (k, traffic[k], alg)
