"""The C-ABI library builds, loads and exports every symbol include/ltpg.h declares (no GPU needed)."""
import ctypes as C
import os
import random

from ltpg_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "ltpg.h")


def test_library_exports_every_declared_symbol(built_lib):
    lib = C.CDLL(built_lib)
    declared = abi.declared_functions(HEADER)
    assert len(declared) >= 30
    missing = [n for n in declared if not hasattr(lib, n)]
    assert not missing, missing
    # the ctypes mirror covers the whole header, and nothing else
    assert sorted(abi.SIGNATURES) == declared


def test_host_hash_matches_oracle_and_python(built_lib):
    import ltpg_gb300
    import oracle
    from kat import hash3
    L, O = ltpg_gb300.lib(), oracle.lib()
    rng = random.Random(3)
    for _ in range(200):
        s, a, b = (rng.getrandbits(64) for _ in range(3))
        assert L.ltpg_hash3(s, a, b) == O.oracle_hash3(s, a, b) == hash3(s, a, b)


def test_create_without_gpu_fails_cleanly(built_lib):
    """On a machine without a GPU, ltpg_create reports an error instead of crashing."""
    import torch
    if torch.cuda.is_available():
        return
    import ltpg_gb300
    try:
        ltpg_gb300.Engine()
    except ltpg_gb300.LtpgError as e:
        assert e.code == abi.ERR_CUDA
    else:
        raise AssertionError("expected LtpgError")


def test_invalid_arguments_rejected(built_lib):
    import ltpg_gb300
    L = ltpg_gb300.lib()
    h = C.c_void_p()
    bad = abi.ConfigC(0, 0, 0, 0, 0, 0)
    assert L.ltpg_create(C.byref(bad), C.byref(h)) == abi.ERR_INVALID
    bad = abi.ConfigC(0, 1, 1024, 64, 0, 0)  # more ops per transaction than supported
    assert L.ltpg_create(C.byref(bad), C.byref(h)) == abi.ERR_INVALID
    p = abi.YcsbParamsC(1, 0, 10, 10, 50, 0, 0.5)  # empty table
    assert L.ltpg_gen_create_ycsb(C.byref(p), C.byref(h)) == abi.ERR_INVALID
    p = abi.YcsbParamsC(1, 100, 10, 10, 50, 0, 1.0)  # theta must be < 1
    assert L.ltpg_gen_create_ycsb(C.byref(p), C.byref(h)) == abi.ERR_INVALID
    q = abi.TpccParamsC(1, 0, 10, 50, 1, 15)  # no warehouses
    assert L.ltpg_gen_create_tpcc(C.byref(q), C.byref(h)) == abi.ERR_INVALID
    # packed order lines: host packing needs its arrays unless there is nothing to pack
    assert L.ltpg_tpcc_pack_lines(None, 5, None) == abi.ERR_INVALID
    assert L.ltpg_tpcc_pack_lines(None, 0, None) == 0
    b = abi.TpccBatchC(1, 0, 0, None, None)
    assert L.ltpg_batch_upload_tpcc_packed(None, 0, C.byref(b), None) == abi.ERR_INVALID
    assert L.ltpg_submit_tpcc_packed_host(None, 0, C.byref(b), None, 0, None) == abi.ERR_INVALID


STRUCTS = {"YcsbBatchC": "ltpg_ycsb_batch", "YcsbParamsC": "ltpg_ycsb_params", "TpccBatchC": "ltpg_tpcc_batch",
           "TpccParamsC": "ltpg_tpcc_params", "ConfigC": "ltpg_config", "LaunchC": "ltpg_launch",
           "PredictorC": "ltpg_predictor_cfg", "ServeCfgC": "ltpg_serve_cfg", "ServeStatsC": "ltpg_serve_stats",
           "StatsC": "ltpg_batch_stats", "BatchInfoC": "ltpg_batch_info"}


def test_ctypes_structs_match_the_header(tmp_path):
    """Every ctypes mirror of an ABI struct has the C struct's size and field
    offsets (gcc compiles the header and prints them)."""
    import subprocess
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "ltpg.h"', "int main(void) {"]
    for py, c in STRUCTS.items():
        lines.append(f'printf("{py} size %zu\\n", sizeof({c}));')
        for name, _ in getattr(abi, py)._fields_:
            lines.append(f'printf("{py} {name} %zu\\n", offsetof({c}, {name}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", os.path.dirname(HEADER), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {tuple(line.split()[:2]): int(line.split()[2]) for line in out if line}
    for py in STRUCTS:
        cls = getattr(abi, py)
        assert got[(py, "size")] == C.sizeof(cls), py
        for name, _ in cls._fields_:
            assert got[(py, name)] == getattr(cls, name).offset, (py, name)


def test_bench_library_exports_its_header(built_lib):
    """The measurement-only library exports what include/ltpg_bench.h declares,
    and the engine library does not carry it."""
    from ltpg_gb300 import build
    bench = C.CDLL(build.BENCH_LIB)
    declared = abi.declared_functions(os.path.join(ROOT, "include", "ltpg_bench.h"))
    assert declared == sorted(abi.BENCH_SIGNATURES)
    assert all(hasattr(bench, n) for n in declared)
    engine = C.CDLL(built_lib)
    assert not any(hasattr(engine, n) for n in declared)
