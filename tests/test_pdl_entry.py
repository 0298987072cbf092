"""Every CUDA kernel of the library begins with pdl_entry().

Kernels are launched with programmatic stream serialisation allowed (gbk::launch in
csrc/gbk_common.cuh), so a kernel may be placed on the SMs while its predecessor on the stream is
still running. Its first statement must therefore wait for the predecessor grid
(griddepcontrol.wait inside pdl_entry) before it touches memory; a kernel without it would read
inputs that are not yet written. This test reads the sources: no GPU is needed.
"""
import pathlib
import re

CSRC = pathlib.Path(__file__).resolve().parents[1] / "deformetrica_code_gb300" / "csrc"


def _kernels(text):
    """(name, first statement of the body) for each __global__ function definition."""
    out = []
    for m in re.finditer(r"__global__\b", text):
        brace = text.index("{", m.end())
        head = text[m.end():brace]
        if ";" in head:  # a declaration, not a definition
            continue
        name = re.findall(r"(\w+)\s*\(", head)
        body = text[brace + 1:]
        first = body.lstrip().split("\n", 1)[0].strip()
        out.append((name[-1] if name else "?", first))
    return out


def test_every_kernel_waits_for_its_predecessor_first():
    files = sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cuh")))
    assert files
    seen = 0
    for f in files:
        for name, first in _kernels(f.read_text()):
            seen += 1
            assert first in ("pdl_entry();", "gbk::pdl_entry();"), f"{f.name}: kernel {name} begins with {first!r}"
    assert seen >= 50


def test_kernels_are_launched_through_the_helper_on_the_deformation_paths():
    # the deformation loops' launch sites use gbk::launch (programmatic dependent launch)
    for fname in ("gbk_pairs.cuh", "gbk_pairs_warp.cuh", "gbk_deform.cu", "gbk_atlas.cu", "gbk_geometry.cu",
                  "gbk_registration.cu", "gbk_geodesic.cu"):
        text = (CSRC / fname).read_text()
        assert "<<<" not in text, f"{fname} still has a <<<>>> launch"
