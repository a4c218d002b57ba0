"""The C-ABI library without compute: it loads, exports every declared
symbol, and its host-only entry points (SVO files, argument checks) behave
like the reference (CPU only)."""
from __future__ import annotations

import json
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = Path(__file__).with_name("golden") / "svo_golden.npz"


def declared_symbols():
    text = "\n".join(p.read_text() for p in (ROOT / "include").glob("*.h"))
    return sorted(set(re.findall(r"XN_API\s+[\w\s\*]+?\b(xn_\w+)\s*\(", text)))


def test_library_exports_every_declared_symbol(built_library):
    import xenodon_gb300 as xg
    names = declared_symbols()
    assert len(names) >= 16
    assert set(names) == set(xg.EXPORTS)
    out = subprocess.run(["nm", "-D", "--defined-only", str(built_library)], capture_output=True, text=True,
                         check=True).stdout
    exported = set(re.findall(r"\bT (xn_\w+)", out))
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    lib = xg.load_library()
    for n in names:
        assert getattr(lib, n) is not None
    assert lib.xn_abi_version() == 1


def test_library_exports_nothing_else(built_library):
    out = subprocess.run(["nm", "-D", "--defined-only", str(built_library)], capture_output=True, text=True,
                         check=True).stdout
    ours = set(re.findall(r"\bT (xn_\w+)", out))
    assert ours == set(declared_symbols())


def test_svo_roundtrip_matches_reference_files(built_library, tmp_path):
    import xenodon_gb300 as xg
    z = np.load(GOLDEN)
    meta = json.loads(bytes(z["meta"]).decode())
    for m in meta[:12]:
        data = bytes(z[m["key"]])
        p = tmp_path / "a.svo"
        p.write_bytes(data)
        nodes, side = xg.svo_load(p)
        assert side == m["stats"]["side"] and nodes.shape[0] == m["stats"]["n_nodes"]
        q = tmp_path / "b.svo"
        xg.svo_save(q, nodes, side)
        assert q.read_bytes() == data


@pytest.mark.parametrize("mutation,msg", [
    (lambda d: b"XNDN-SVX" + d[8:], "Invalid format id"),
    (lambda d: d[:-4], "File size does not match"),
    (lambda d: d + b"\0" * 40, "File size does not match"),
    (lambda d: d[:10], "truncated header"),
])
def test_malformed_svo_files_are_rejected(built_library, tmp_path, mutation, msg):
    import xenodon_gb300 as xg
    z = np.load(GOLDEN)
    meta = json.loads(bytes(z["meta"]).decode())
    p = tmp_path / "bad.svo"
    p.write_bytes(mutation(bytes(z[meta[0]["key"]])))
    with pytest.raises(xg.XenodonError) as e:
        xg.svo_load(p)
    assert msg in str(e.value)


def test_missing_svo_file(built_library, tmp_path):
    import xenodon_gb300 as xg
    with pytest.raises(xg.XenodonError) as e:
        xg.svo_load(tmp_path / "nope.svo")
    assert e.value.code == xg.XN_ERR_IO


def test_create_without_gpu_fails_cleanly(built_library):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import xenodon_gb300 as xg
    with pytest.raises(xg.XenodonError) as e:
        xg.Context(0)
    assert e.value.code in (xg.XN_ERR_CUDA, xg.XN_ERR_ARG)


def test_null_arguments_are_rejected(built_library):
    import ctypes
    import xenodon_gb300 as xg
    lib = xg.load_library()
    assert lib.xn_create(0, 0, None) == xg.XN_ERR_ARG
    assert b"NULL" in lib.xn_last_error()
    assert lib.xn_render(None, None, 0, None, None, None, None, None) == xg.XN_ERR_ARG
    assert lib.xn_destroy(None) == xg.XN_OK
    assert lib.xn_volume_release(None) == xg.XN_OK
    out = ctypes.POINTER(ctypes.c_uint32)()
    st = xg.BuildStats()
    assert lib.xn_build_svo(None, None, 1, 1, 1, 0, 0, 0.0, ctypes.byref(out), ctypes.byref(st)) == xg.XN_ERR_ARG


# ctypes mirror -> the header's typedef name
MIRRORS = {"Camera": "xn_camera", "Rect": "xn_rect", "Params": "xn_params", "VolumeInfo": "xn_volume_info",
           "Job": "xn_job", "BatchConfig": "xn_batch_config", "ServerConfig": "xn_server_config",
           "ServerStats": "xn_server_metrics", "BuildStats": "xn_build_stats"}


def test_ctypes_structures_match_the_header(tmp_path):
    """Size and every field offset of the Python mirrors equal the C
    compiler's for include/xenodon.h (a field added on one side only would
    shift what the library reads)."""
    import ctypes
    import xenodon_gb300 as xg
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "xenodon.h"', "int main(void) {"]
    expect = []
    for py, c in MIRRORS.items():
        cls = getattr(xg, py)
        lines.append(f'printf("{c} %zu\\n", sizeof({c}));')
        expect.append(f"{c} {ctypes.sizeof(cls)}")
        for name, _ in cls._fields_:
            lines.append(f'printf("{c}.{name} %zu\\n", offsetof({c}, {name}));')
            expect.append(f"{c}.{name} {getattr(cls, name).offset}")
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    got = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    assert [g for g in got if g] == expect
