"""bench.py's launch accounting (kernel names, blind-rotation launches per
step for the roofline traffic, eager launch count) restates the engine's
automatic split-FP32 shape (launch_auto_fp32 in csrc/bootstrap.cu, rule in
include/tfhe_gpu.h): whole waves of 6 per SM on shape 10; a remainder of at
most one per two SMs on the cluster spread kernel, at most 1 per SM on the
spread kernel, 2 per SM on the pair kernel, at most 4 per SM as one shape-9
wave, else one more shape-10 wave.  CPU only."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

bench = pytest.importorskip("bench")

PAIRS = "k_blind_rotate_ring<float,2,6,3,4,inline,nb2>"
BATCHED = "k_blind_rotate_ring<float,2,4,3,4,inline,nb3>"
SPREAD = "k_blind_rotate_spread<3>"
SPREAD2 = "k_blind_rotate_spread2<3>"
PAIR2 = "k_blind_rotate_pair<float,2,2,3,4>"


@pytest.mark.parametrize("batch,want", [
    (1, [SPREAD2 + " x 1"]),
    (76, [SPREAD2 + " x 76"]),
    (77, [SPREAD + " x 77"]),
    (152, [SPREAD + " x 152"]),
    (153, [PAIR2 + " x 153"]),
    (304, [PAIR2 + " x 304"]),
    (305, [BATCHED + " x 305"]),
    (608, [BATCHED + " x 608"]),
    (609, [PAIRS]),
    (912, [PAIRS]),
    (913, [PAIRS + " x 912", SPREAD2 + " x 1"]),
    (1064, [PAIRS + " x 912", SPREAD + " x 152"]),
    (1216, [PAIRS + " x 912", PAIR2 + " x 304"]),
    (1520, [PAIRS + " x 912", BATCHED + " x 608"]),
    (1521, [PAIRS]),
    (4096, [PAIRS + " x 3648", BATCHED + " x 448"]),
])
def test_automatic_shape_launches(batch, want):
    assert bench.blind_rotate_kernels("split_fp32", 0, batch) == want


def test_fixed_order_shape_has_no_pair_kernel():
    assert bench.blind_rotate_kernels("split_fp32", 15, 200) == [SPREAD + " x 200"]
    assert bench.blind_rotate_kernels("split_fp32", 15, 912 + 60) == [PAIRS + " x 912", SPREAD2 + " x 60"]
    assert bench.blind_rotate_kernels("split_fp32", 15, 4096) == bench.blind_rotate_kernels("split_fp32", 0, 4096)


def test_explicit_shapes_and_other_set():
    assert bench.blind_rotate_kernels("split_fp32", 9, 100) == [BATCHED]
    assert bench.blind_rotate_kernels("split_fp32", 10, 100) == [PAIRS]
    assert bench.blind_rotate_kernels("split_fp32", 14, 5) == [SPREAD]
    assert bench.blind_rotate_kernels("split_fp32", 16, 5) == [SPREAD2]
    assert bench.blind_rotate_kernels("split_fp32", 12, 5) == [PAIR2]
    assert bench.blind_rotate_kernels("split_fp32", 10, 100, l=2) == ["k_blind_rotate_ring<float,2,6,2,4,inline,nb2>"]
    assert bench.blind_rotate_kernels("fp64", 3, 100) == ["k_external_product<double,1,BlindRotate,3,3>"]
    assert bench.blind_rotate_kernels("fp64", 0, 153) == ["k_external_product<double,1,BlindRotate,3,3>"]
    assert bench.blind_rotate_kernels("fp64", 0, 152) == ["k_blind_rotate_spread2_f64<3>"]
    assert bench.blind_rotate_kernels("fp64", 16, 4096) == ["k_blind_rotate_spread2_f64<3>"]


def test_shared_memory_roofline_counts_each_kernel_part():
    kernels = bench.blind_rotate_kernels("split_fp32", 0, 4096)
    r = bench.smem_roofline(kernels, 4096, 31.0, {"sm_mhz": 2000.0})
    want = 3648 * 1.58e9 / 912 + 448 * 0.74e9 / 448
    assert abs(r["wavefronts_per_step"] - want) < 1.0
    assert abs(r["achieved"] - want / 0.031 / 1e9) < 1e-6
    assert abs(r["peak"] - 152 * 2000.0 / 1000.0) < 1e-9
    # one whole-batch launch of a counted kernel
    r = bench.smem_roofline([PAIRS], 912, 6.6, None)
    assert abs(r["wavefronts_per_step"] - 1.58e9) < 1.0
    # a step with a kernel that has no count gives no figure
    assert bench.smem_roofline(bench.blind_rotate_kernels("split_fp32", 0, 100), 100, 1.3, None) is None
