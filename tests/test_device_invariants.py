"""Invariants of the device code that hold by construction, checked on the CPU.

A host program compiled by nvcc against csrc/ozaki.cuh (its __host__ __device__
functions run on the host) checks:
  * exactness of the exact-slice products: for every inner dimension K that the
    library uses (1..1024), the slice width B of cfg_for_k(K) keeps each weight group
    m <= 3 (at most 4 slice pairs) of the FP32 tensor-core accumulation below 2^24,
    i.e. 4 (2^B - 1)^2 K < 2^24, so those groups are exact integers, and the slices
    carry at least 48 bits;
  * the tensor-core image layout: tc_index maps (line, k) of a slice padded to
    tc_lines(N) lines and ldk columns one-to-one onto [0, tc_slice_elems), and the
    16-deep chunk of any 128 consecutive lines starting at a multiple of 128 is one
    contiguous range of 2048 elements (what one bulk copy moves);
  * the submatrix Metropolis kernels' dynamic shared memory fits one CTA for every N and
    spin count the library takes (a program linked against kernels_submatrix.cu).
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "dqmc-framework_gb300", "csrc")

PROGRAM = r"""
#include <cstdio>
#include <vector>
#include "ozaki.cuh"
using namespace dqmc::ozaki;

int main() {
  int bad = 0;
  for (int K = 1; K <= 1024; ++K) {
    const SliceCfg c = cfg_for_k(K);
    const double top = (double)((1 << c.bits) - 1);
    if (!(4.0 * top * top * K < 16777216.0)) { std::printf("K=%d: group sums reach 2^24\n", K); ++bad; }
    if (c.bits * c.slices < 48 || c.slices > kMaxSlices) { std::printf("K=%d: %d x %d bits\n", K, c.slices, c.bits); ++bad; }
  }
  const int Ns[] = {4, 36, 64, 81, 100, 144, 256, 289, 576, 1024};
  for (int N : Ns) {
    const int ldk = (N + 15) / 16 * 16, lines = tc_lines(N), nlb = lines / 8;
    const size_t total = tc_slice_elems(N, ldk);
    std::vector<unsigned char> seen(total, 0);
    for (int line = 0; line < lines; ++line)
      for (int k = 0; k < ldk; ++k) {
        const long long i = tc_index(line, k, nlb);
        if (i < 0 || (size_t)i >= total || seen[i]) { std::printf("N=%d: (%d,%d) -> %lld\n", N, line, k, i); ++bad; break; }
        seen[i] = 1;
      }
    for (int l0 = 0; l0 < lines; l0 += 128)
      for (int k0 = 0; k0 < ldk; k0 += 16) {
        long long lo = tc_index(l0, k0, nlb), hi = lo;
        for (int l = l0; l < l0 + 128; ++l)
          for (int k = k0; k < k0 + 16; ++k) {
            const long long i = tc_index(l, k, nlb);
            lo = i < lo ? i : lo;
            hi = i > hi ? i : hi;
          }
        if (hi - lo + 1 != 2048 || lo % 2048 != 0) { std::printf("N=%d: chunk (%d,%d) not contiguous\n", N, l0, k0); ++bad; }
      }
  }
  std::printf("%s\n", bad ? "FAIL" : "OK");
  return bad ? 1 : 0;
}
"""


def test_slice_exactness_and_image_layout(tmp_path):
    nvcc = shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else None)
    if nvcc is None:
        pytest.skip("nvcc not available")
    src = tmp_path / "invariants.cu"
    src.write_text(PROGRAM)
    exe = tmp_path / "invariants"
    subprocess.run([nvcc, "-std=c++17", "-O1", "-I", CSRC, str(src), "-o", str(exe)], check=True, timeout=300)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip().endswith("OK"), r.stdout[-2000:]


def _src(name):
    return open(os.path.join(CSRC, name), encoding="utf-8").read()


def test_stabilization_and_flush_slice_widths():
    """The widths the stabilization products and the Metropolis flushes are compiled with
    (read from the sources) keep their groups exact: the stabilization's groups m <= 3 below
    2^24 for K up to the largest N it takes (256 for 8 x 7 bits, kMaxOzN for 9 x 6); the
    flush reads every group through the 1.5 * 2^23 bias, so all of them, with up to S pairs,
    must stay below 2^22 for K = the block size."""
    import re

    stab = _src("kernels_stab_oz.cu")
    s56 = re.search(r"#define ZGEMM56 zgemm_tc_kernel<(\d+), (\d+),", stab)
    s54 = re.search(r"#define ZGEMM54 zgemm_tc_kernel<(\d+), (\d+),", stab)
    assert s56 and s54
    assert re.search(r"if \(maxN > 256\) ZGEMM54", stab)
    kmax_oz = int(re.search(r"constexpr int kMaxOzN = (\d+);", _src("batch.cu")).group(1))
    for (S, B), kmax in (((int(s56.group(1)), int(s56.group(2))), 256), ((int(s54.group(1)), int(s54.group(2))), kmax_oz)):
        assert 4 * (2 ** B - 1) ** 2 * kmax < 2 ** 24, (S, B, kmax)
        assert S * B >= 54  # the accuracy class of an FP64 product
    sub = _src("kernels_submatrix.cu")
    S, B = map(int, re.search(r"constexpr int OZS = (\d+), OZB = (\d+);", sub).groups())
    KB = int(re.search(r"constexpr int KB = (\d+);", sub).group(1))
    assert S * (2 ** B - 1) ** 2 * KB < 2 ** 22


SMEM_PROGRAM = r"""
#include <cstdio>
namespace dqmc {
size_t submatrix_smem_bytes(int N, int S);
size_t submatrix_block_smem_bytes(int S);
size_t submatrix_flush_smem_bytes(int N);
}
int main() {
  // the opt-in dynamic shared memory of one CTA on sm_100-class GPUs (227 KB), less 2 KB for
  // the kernels' static shared memory
  const size_t limit = 232448 - 2048;
  int bad = 0;
  for (int S = 1; S <= 2; ++S) {
    for (int N = 1; N <= 1024; ++N) {
      if (dqmc::submatrix_smem_bytes(N, S) > limit) { std::printf("fused N=%d S=%d\n", N, S); ++bad; break; }
      if (dqmc::submatrix_flush_smem_bytes(N) > limit) { std::printf("flush N=%d\n", N); ++bad; break; }
    }
    if (dqmc::submatrix_block_smem_bytes(S) > limit) { std::printf("block S=%d\n", S); ++bad; }
  }
  std::printf("%s\n", bad ? "FAIL" : "OK");
  return bad ? 1 : 0;
}
"""


def test_submatrix_kernels_fit_in_shared_memory(tmp_path):
    """The submatrix Metropolis kernels' dynamic shared memory (operand buffers, block state,
    G staging, exponents), as the launches size it, fits one CTA for every N <= 1024 and both
    spin counts; the functions are the library's own, linked from kernels_submatrix.cu."""
    nvcc = shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else None)
    if nvcc is None:
        pytest.skip("nvcc not available")
    src = tmp_path / "smem.cu"
    src.write_text(SMEM_PROGRAM)
    exe = tmp_path / "smem"
    subprocess.run([nvcc, "-std=c++17", "-O1", "-gencode", "arch=compute_103a,code=sm_103a", "-I", CSRC, str(src),
                    os.path.join(CSRC, "kernels_submatrix.cu"), "-o", str(exe)], check=True, timeout=600)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and r.stdout.strip().endswith("OK"), r.stdout
