"""The C++ drop-in adapters compile against the reference's own headers: the
dense-field generator adapter instantiates BlockTreeFieldService<3>::interpolateWith
(include/s3dmm/BlockTreeFieldService.hpp:118-145) for both dense containers."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
# the reference headers as staged by `make -C oracle stage REFERENCE=<root>`
TREE = ROOT / "oracle" / "_ref" / "tree"

SRC = r'''
#include "s3dmm/BlockTreeFieldService.hpp"
#include "DenseFieldInterpolatorGb300.hpp"
using S = s3dmm::BlockTreeFieldService<3>;
template void S::interpolateWith<s3dmm::DenseFieldInterpolatorGb300<std::vector<float>&>>(
    s3dmm::Vec2<s3dmm::dfield_real>&, std::vector<float>&, unsigned int, unsigned int, const BlockId&,
    s3dmm::FieldTimestamps*) const;
template void S::interpolateWith<s3dmm::DenseFieldInterpolatorGb300<s3dmm::Gb300DenseField&>>(
    s3dmm::Vec2<s3dmm::dfield_real>&, s3dmm::Gb300DenseField&, unsigned int, unsigned int, const BlockId&,
    s3dmm::FieldTimestamps*) const;
'''


def test_dense_field_interpolator_adapter_compiles(tmp_path):
    if not (TREE / "include" / "s3dmm" / "BlockTreeFieldService.hpp").exists():
        pytest.skip("reference headers not staged")
    from revise_gb300.build import cuda_home
    cuda_inc = cuda_home() / "include"
    if not cuda_inc.exists() or not shutil.which("g++"):
        pytest.skip("no toolchain")
    src = tmp_path / "adapter_check.cpp"
    src.write_text(SRC)
    cmd = ["g++", "-std=c++20", "-fsyntax-only", "-DS3DMM_REAL_TYPE=float", "-DS3DMM_ENABLE_CUDA",
           "-DS3DMM_PROGRESS_REPORT", f"-I{ROOT / 'oracle' / 'shims_cpu'}", f"-I{ROOT / 'oracle' / 'shims'}", f"-I{TREE / 'include'}",
           f"-I{ROOT / 'include'}", f"-I{ROOT / 'revise_gb300' / 'adapters'}", f"-I{cuda_inc}", str(src)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


def test_renderer_and_worker_adapters_compile(tmp_path):
    """DenseFieldRendererGb300 and VsWorkerGb300 against the reference's renderer and worker interfaces
    (include/s3dmm_cuda/DenseFieldRenderer_cu.hpp, include/s3vs/VsWorkerInterface.hpp); the program that
    runs them on the GPU (tests/adapters/adapter_check.cpp) is syntax-checked here too."""
    if not (TREE / "include" / "s3vs" / "VsWorkerInterface.hpp").exists():
        pytest.skip("reference headers not staged")
    from revise_gb300.build import cuda_home
    cuda_inc = cuda_home() / "include"
    if not cuda_inc.exists() or not shutil.which("g++"):
        pytest.skip("no toolchain")
    cmd = ["g++", "-std=c++20", "-fsyntax-only", "-DS3DMM_REAL_TYPE=float", "-DS3DMM_ENABLE_CUDA",
           "-DS3DMM_PROGRESS_REPORT", f"-I{ROOT / 'oracle' / 'shims_cuda'}", f"-I{ROOT / 'oracle' / 'shims'}",
           f"-I{TREE / 'include'}", f"-I{TREE / 'src' / 's3dmm_cuda'}", f"-I{ROOT / 'include'}",
           f"-I{ROOT / 'revise_gb300' / 'adapters'}", f"-I{cuda_inc}", str(ROOT / "tests" / "adapters" / "adapter_check.cpp")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
