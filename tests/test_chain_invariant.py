"""Chained launches (programmatic dependent launch inside CUDA-graph capture)
are only correct for kernels that wait for the kernel before them before they
touch global memory: every kernel that launch_chained launches must start with
chain_enter(). Checked on the CUDA sources, without a GPU."""
import os
import re

from pipeline_gb300 import build as B


def _sources():
    out = {}
    for f in sorted(os.listdir(B.CSRC)):
        if f.endswith((".cu", ".cuh")):
            out[f] = open(os.path.join(B.CSRC, f)).read()
    return out


def _chained_names(srcs):
    names = set()
    for text in srcs.values():
        for m in re.finditer(r"launch_chained\(\s*([A-Za-z_]\w*)", text):
            if m.group(1) not in ("void",):  # the template's own declaration
                names.add(m.group(1))
    # `auto k = kernel<...>;` aliases passed as `k`
    aliases = {}
    for text in srcs.values():
        for m in re.finditer(r"auto\s+(\w+)\s*=\s*([A-Za-z_]\w*)\s*<", text):
            aliases[m.group(1)] = m.group(2)
    return {aliases.get(n, n) for n in names if n != "kernel"}


def _kernel_bodies(srcs, name):
    """The first statements of every __global__ definition of `name`."""
    bodies = []
    for text in srcs.values():
        for m in re.finditer(r"__global__[^;{]*?\b" + re.escape(name) + r"\s*\(", text):
            brace = text.index("{", m.end())
            bodies.append(text[brace + 1:brace + 200])
    return bodies


def test_every_chained_kernel_waits_first():
    srcs = _sources()
    names = _chained_names(srcs)
    assert len(names) >= 15, names
    for name in sorted(names):
        bodies = _kernel_bodies(srcs, name)
        assert bodies, f"no __global__ definition found for {name}"
        for body in bodies:
            first = body.strip().split(";")[0].strip()
            assert first == "chain_enter()", f"{name} starts with {first!r}"


def test_chain_enter_waits_before_it_releases():
    text = open(os.path.join(B.CSRC, "common.cuh")).read()
    m = re.search(r"void chain_enter\(\)\s*\{(.*?)\}", text, re.S)
    assert m
    body = m.group(1)
    assert body.index("chain_wait()") < body.index("chain_release()")
    assert "griddepcontrol.wait" in text and "griddepcontrol.launch_dependents" in text


def test_chained_launches_only_inside_graph_capture():
    text = open(os.path.join(B.CSRC, "kernels.cuh")).read()
    m = re.search(r"launch_chained\(void \(\*kernel\)\(P\.\.\.\).*?\n\}", text, re.S)
    assert m
    assert "chained_launches() && stream_capturing(s)" in m.group(0)
