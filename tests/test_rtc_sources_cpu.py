"""The generated constraint kernels compile under NVRTC as the library compiles them (the same
in-memory headers and options: sm_103a, C++17), on the CPU. NVRTC sees no system headers, so a
fixed-width type the prelude does not define fails here rather than on the device."""
import pytest

from proving_gb300 import framework as fw
from test_mask_offsets_cpu import window_air

nvrtc = pytest.importorskip("cuda.bindings.nvrtc")


def _relation_lookup_air(e):
    # a relation entry (with the fraction kernel beside the composition kernel)
    e.add_to_relation("lookup", -1, [e.next_trace_mask()])
    e.finalize_logup()


def _compile(source: str):
    names = ["field.cuh", "rows.cuh"]
    headers = [fw._header(n).encode() for n in names]
    err, prog = nvrtc.nvrtcCreateProgram(source.encode(), b"air.cu", len(names), headers,
                                         [n.encode() for n in names])
    assert err == nvrtc.nvrtcResult.NVRTC_SUCCESS
    opts = [b"--gpu-architecture=sm_103a", b"-std=c++17"]
    (rc,) = nvrtc.nvrtcCompileProgram(prog, len(opts), opts)
    err, size = nvrtc.nvrtcGetProgramLogSize(prog)
    log = b" " * size
    nvrtc.nvrtcGetProgramLog(prog, log)
    nvrtc.nvrtcDestroyProgram(prog)
    return rc, log.decode(errors="replace")


@pytest.mark.parametrize("name,make", [
    ("wide_fib", lambda: fw.compile_air("wide_fib", fw.wide_fib_air, 5)),
    ("single_lookup", lambda: fw.compile_air("single_lookup", fw.single_lookup_air)),
    ("window", lambda: fw.compile_air("window", window_air)),
    ("lookup_relation", lambda: fw.compile_air("lookup_rel", _relation_lookup_air)),
])
def test_generated_source_compiles_under_nvrtc(name, make):
    rc, log = _compile(make().source)
    assert rc == nvrtc.nvrtcResult.NVRTC_SUCCESS, log


def test_split_source_with_offsets_compiles_under_nvrtc(monkeypatch):
    monkeypatch.setattr(fw, "_SINGLE_LINES", 4)
    monkeypatch.setattr(fw, "_CHUNK_NODES", 2)
    air = fw.compile_air("window", window_air)
    assert "cs_air_group1(" in air.source
    rc, log = _compile(air.source)
    assert rc == nvrtc.nvrtcResult.NVRTC_SUCCESS, log
