"""The C-ABI library loads, exports every entry point the header declares,
and refuses cleanly where no GPU is present. CPU only."""

import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols(header):
    src = open(os.path.join(ROOT, "include", header)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(zc_[a-z0-9_]+)\s*\(", src)))


def test_header_exports(zc):
    from zeno_gb300 import serve

    lib = ctypes.CDLL(zc.LIB_PATH)
    headers = sorted(f for f in os.listdir(os.path.join(ROOT, "include")) if f.endswith(".h"))
    assert headers == ["zeno_cuda.h", "zeno_cuda_serve.h"]
    core, srv = declared_symbols("zeno_cuda.h"), declared_symbols("zeno_cuda_serve.h")
    assert len(core) >= 25 and len(srv) == 6
    missing = [n for n in core + srv if not hasattr(lib, n)]
    assert not missing, missing
    assert sorted(zc.EXPORTS) == core
    assert sorted(serve.EXPORTS) == srv


def test_capacity_planning(zc):
    """mem.rs retargeted to HBM: 33 qubits f64 / 34 f32 in 0.75 x 284208 MiB."""
    hbm = 284208 * (1 << 20)
    budget = int(hbm * 0.75)
    assert zc.max_qubits(budget, 64) == 33
    assert zc.max_qubits(budget, 32) == 34
    assert zc.state_bytes(30, 64) == 16 << 30
    assert zc.max_qubits(24 << 30, 64) == 30 and zc.max_qubits(24 << 30, 32) == 31


def test_env_budget_override(zc, monkeypatch):
    """ZENO_MEM_BYTES pretends to be a smaller machine (src/mem.rs:9-16); the
    budget is 0.75 of it: 16 GiB -> 12 GiB -> 29 qubits f64, 30 f32, as
    tests/cli.rs:126-153 expects of `zeno info`."""
    monkeypatch.setenv("ZENO_MEM_BYTES", str(16 << 30))
    assert zc.device_memory() == 16 << 30
    budget = zc.device_budget()
    assert budget == 12 << 30
    assert zc.max_qubits(budget, 64) == 29 and zc.max_qubits(budget, 32) == 30
    assert zc.state_bytes(29, 64) == (1 << 29) * 16 and zc.state_bytes(30, 64) == (1 << 30) * 16


def _have_gpu():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_have_gpu(), reason="checks the no-GPU refusal path")
def test_create_without_gpu_fails_loudly(zc):
    with pytest.raises(zc.ZenoCudaError) as e:
        zc.CudaBackend(4, 64)
    assert e.value.code in (zc.ZC_ERR_UNSUPPORTED, zc.ZC_ERR_CUDA)


def test_invalid_arguments_rejected_before_device(zc, monkeypatch):
    monkeypatch.setenv("ZENO_MEM_BYTES", str(1 << 20))
    with pytest.raises(zc.ZenoCudaError):
        zc.CudaBackend(4, 48)  # bad precision


def test_info_capacity_rows(zc, monkeypatch):
    """The info table's rows come from the same capacity math (no device needed
    for the rows themselves)."""
    from zeno_gb300 import info

    budget = int(284208 * (1 << 20) * 0.75)
    f64, f32 = info.capacity(budget, 64), info.capacity(budget, 32)
    assert (f64["max_qubits"], f32["max_qubits"]) == (33, 34)
    assert f64["state_bytes"] == 128 << 30 and f64["next_qubit_bytes"] == 256 << 30
    assert info.human(128 << 30) == "128.0 GiB" and info.human(512) == "512 B"


def test_noise_model_validated_by_the_abi(zc, monkeypatch):
    """zc_run validates a non-trivial noise model before anything else, as
    run_inner does (src/exec.rs:347-351; NoiseModel::validate,
    src/noise.rs:77-87): every field in [0, 1], NaN rejected, 1 allowed.
    The Python wrapper's own check is bypassed to reach the C ABI."""
    from zeno_gb300 import circuit as C

    monkeypatch.setattr(zc.NoiseModel, "validate", lambda self: None)
    c = C.Circuit(2)
    c.h(0).cx(0, 1).measure_all()
    p = c.to_program()
    for field, bad in (("depolarizing_1q", -0.1), ("depolarizing_1q", 1.5), ("depolarizing_1q", float("nan")),
                       ("readout_flip_1to0", 1.0001)):
        with pytest.raises(zc.ZenoCudaError, match=field + r" = .* is not a probability in \[0, 1\]"):
            zc.run(p, shots=16, seed=1, precision=32, noise=zc.NoiseModel(**{field: bad}))
    # valid models pass validation (without a GPU the run then fails on the device)
    for ok in (zc.NoiseModel(depolarizing_1q=1.0), zc.NoiseModel(bit_flip=0.0, phase_flip=0.5)):
        try:
            zc.run(p, shots=16, seed=1, precision=32, noise=ok)
        except zc.ZenoCudaError as e:
            assert "not a probability" not in str(e)


@pytest.mark.parametrize("lang, std", [("c", "-std=c99"), ("c++", "-std=c++17")])
def test_headers_compile_as_plain_c_and_cpp(tmp_path, lang, std):
    """The boundary is a C ABI: both public headers compile alone, warning
    free and pedantic, as C99 (what a Rust or cgo binding parses) and C++."""
    import shutil
    import subprocess

    cc = shutil.which("gcc" if lang == "c" else "g++")
    if cc is None:
        pytest.skip("no host compiler")
    src = tmp_path / "hdr.c"
    src.write_text('#include "zeno_cuda.h"\n#include "zeno_cuda_serve.h"\nint main(void) { return 0; }\n')
    subprocess.run([cc, std, "-Wall", "-Wextra", "-pedantic", "-Werror", "-x", lang, "-I" + os.path.join(ROOT, "include"),
                    "-c", str(src), "-o", str(tmp_path / "hdr.o")], check=True)


def test_ctypes_mirrors_match_the_c_layouts(zc, tmp_path):
    """Every ctypes mirror of a header struct has the C struct's size and each
    field's C offset (a C program built from the mirrors prints them; a field
    the C struct lacks fails to compile)."""
    import ctypes as C
    import shutil
    import subprocess

    from zeno_gb300 import serve

    cc = shutil.which("gcc")
    if cc is None:
        pytest.skip("no host compiler")
    pairs = [("zc_device", zc.DeviceC), ("zc_counters", zc.Counters), ("zc_kernel_stat", zc.KernelStat),
             ("zc_instr", zc.Instr), ("zc_compile_options", zc.CompileOptions), ("zc_op_view", zc.OpView),
             ("zc_program_info", zc.ProgramInfo), ("zc_noise", zc.NoiseC), ("zc_run_options", zc.RunOptions),
             ("zc_run_result", zc.RunResultC), ("zc_server_options", serve.ServerOptions),
             ("zc_server_status", serve.ServerStatus), ("zc_arith_peaks", zc.ArithPeaksC)]
    lines, want = [], []
    for cname, py in pairs:
        lines.append('printf("%%zu\\n", sizeof(%s));' % cname)
        want.append(C.sizeof(py))
        for f in py._fields_:
            lines.append('printf("%%zu\\n", offsetof(%s, %s));' % (cname, f[0]))
            want.append(getattr(py, f[0]).offset)
    src = tmp_path / "layout.c"
    src.write_text('#include <stddef.h>\n#include <stdio.h>\n#include "zeno_cuda.h"\n#include "zeno_cuda_serve.h"\n'
                   "int main(void) {\n" + "\n".join(lines) + "\nreturn 0;\n}\n")
    exe = str(tmp_path / "layout")
    subprocess.run([cc, "-std=c99", "-I" + os.path.join(ROOT, "include"), str(src), "-o", exe], check=True)
    got = [int(x) for x in subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split()]
    assert got == want


def test_build_targets_sm_103a_only():
    """Every translation unit is compiled for sm_103a alone (no other
    architecture, no PTX for JIT), with line info for the profiler, and host
    code without FMA contraction (bit-identical host arithmetic on x86-64
    and aarch64)."""
    from zeno_gb300 import build

    flags = build.NVCC_FLAGS
    archs = [flags[i + 1] for i, f in enumerate(flags) if f == "-gencode"]
    assert archs == ["arch=compute_103a,code=sm_103a"]
    assert "-lineinfo" in flags and "-ffp-contract=off" in flags
    assert not any(f.startswith(("-arch", "--gpu-architecture")) for f in flags)
