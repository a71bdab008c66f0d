"""CPU test of the recipe that makes the reference program buildable with
CUDA 13 (oracle/ref_cuda13.sed, applied by `make -C oracle ref`): every
edit it names must apply, it must leave the kernels and their arithmetic
untouched, and the constructs CUDA 13 / gcc reject must be gone. Skipped
where the reference's source is absent."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_SRC = "/root/reference/cuDebye-v15.cu"


@pytest.fixture(scope="module")
def edited():
    if not os.path.exists(REF_SRC):
        pytest.skip("the reference's source is not here")
    out = subprocess.run(["sed", "-f", os.path.join(ROOT, "oracle", "ref_cuda13.sed"),
                          REF_SRC], capture_output=True, check=True).stdout
    with open(REF_SRC, "rb") as f:
        orig = f.read()
    return orig.decode("latin-1").splitlines(), out.decode("latin-1").splitlines()


def test_recipe_applies_every_edit(edited):
    orig, new = edited
    text = "\n".join(new)
    assert "thrust::identity" not in text
    assert all("long long unsigned int(" not in l for l in new)
    assert not any(l.startswith("void main(") for l in new)
    assert any(l.startswith("int main(int argc, char* argv[])") for l in new)
    assert "prop.clockRate" not in text and "prop.kernelExecTimeoutEnabled" not in text
    assert "#include <cuda/std/functional>" in text
    # one line added (the include), two removed (the removed properties)
    assert len(new) == len(orig) + 1 - 2


def test_recipe_leaves_the_kernels_alone(edited):
    orig, new = edited

    def kernels(lines):
        out, keep = [], False
        for l in lines:
            if l.startswith("__global__"):
                keep = True
            if keep:
                out.append(l)
            if keep and l.startswith("}"):
                keep = False
        return out

    k_orig, k_new = kernels(orig), kernels(new)
    assert len(k_orig) > 50
    assert k_orig == k_new
