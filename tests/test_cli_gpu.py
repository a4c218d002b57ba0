"""`xenodon render --headless` and `xenodon convert` end to end on the GPU:
files in, files out, checked against the reference builder's golden bytes and
the oracle's images."""
from __future__ import annotations

import json
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

import oracle
from xenodon_gb300 import CLI_PATH

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).with_name("golden") / "svo_golden.npz"


def run(*args, cwd):
    p = subprocess.run([str(CLI_PATH), *map(str, args)], capture_output=True, text=True, cwd=cwd, timeout=300)
    return p.returncode, p.stdout


def png_pixels(path) -> np.ndarray:
    from pngdec import decode
    return decode(Path(path).read_bytes())


@pytest.mark.parametrize("svo_type,flag", [("sparse", []), ("rope", ["--rope"]), ("dag", ["--dag"])])
def test_convert_writes_the_reference_bytes(ctx, tmp_path, svo_type, flag):
    import xenodon_gb300 as xg
    z = np.load(GOLDEN)
    meta = json.loads(bytes(z["meta"]).decode())
    m = next(m for m in meta if m["grid"] == "blob13x11x16" and m["type"] == svo_type and m["threshold"] == 0
             and m["heuristic"] == "chan-diff")
    xg.tiff_save(tmp_path / "in.tif", z["grid__blob13x11x16"])
    rc, out = run("convert", *flag, "in.tif", "out.svo", cwd=tmp_path)
    assert rc == 0, out
    assert (tmp_path / "out.svo").read_bytes() == bytes(z[m["key"]])
    st = m["stats"]
    assert f" Total nodes: {st['total_nodes']} (" in out
    assert f" Unique nodes: {st['n_nodes']} (" in out
    assert f" Total leaves: {st['total_leaves']}\n" in out
    assert f" Unique leaves: {st['unique_leaves']}\n" in out
    assert f" Depth: {st['depth']}\n" in out
    assert f" Dimensions: {st['side']}x{st['side']}x{st['side']}\n" in out
    perfect = (8 ** st["depth"] - 1) // 9
    assert f" Perfect tree nodes: {perfect}\n" in out


def test_convert_streamed_writes_the_reference_bytes(ctx, tmp_path):
    """`convert --streamed` (one top-level octant at a time on the device)
    writes the reference builder's own bytes for every sparse golden file."""
    import xenodon_gb300 as xg
    z = np.load(GOLDEN)
    meta = json.loads(bytes(z["meta"]).decode())
    done = 0
    for m in meta:
        if m["type"] != "sparse":
            continue
        xg.tiff_save(tmp_path / "in.tif", z["grid__" + m["grid"]])
        flag = ["--chan-diff", str(m["threshold"])] if m["heuristic"] == "chan-diff" else \
            ["--std-dev", repr(float(m["threshold"]))]
        rc, out = run("convert", "--streamed", *flag, "in.tif", "out.svo", cwd=tmp_path)
        assert rc == 0, out
        assert (tmp_path / "out.svo").read_bytes() == bytes(z[m["key"]]), m["key"]
        assert f" Unique nodes: {m['stats']['n_nodes']} (" in out
        done += 1
    assert done >= 5
    rc, out = run("convert", "--streamed", "--rope", "in.tif", "out.svo", cwd=tmp_path)
    assert rc == 1 and "--streamed builds a sparse tree" in out


def test_convert_std_dev(ctx, tmp_path):
    import xenodon_gb300 as xg
    z = np.load(GOLDEN)
    meta = json.loads(bytes(z["meta"]).decode())
    m = next(m for m in meta if m["grid"] == "smooth17x13x11" and m["type"] == "rope" and m["heuristic"] == "std-dev")
    xg.tiff_save(tmp_path / "in.tif", z["grid__smooth17x13x11"])
    rc, out = run("convert", "--rope", "--std-dev", str(m["threshold"]), "in.tif", "out.svo", cwd=tmp_path)
    assert rc == 0, out
    assert (tmp_path / "out.svo").read_bytes() == bytes(z[m["key"]])


CAMS = [((0, 0, -0.8660254), (0, 1, 0), (0.5, 0.5, 2.5)),
        ((0.3, -0.1, -0.95), (0, 1, -0.105), (0.2, 0.7, 2.2)),
        ((0.6, 0.3, 0.74), (-0.2, 0.95, 0.0), (0.45, 0.55, 0.5))]


def _write_cams(path):
    from xenodon_gb300 import cameras
    cameras.write_script(path, CAMS)


@pytest.mark.parametrize("shader", ["dda", "svo-naive", "esvo", "svo-df", "svo-rope"])
def test_render_frames_match_oracle(ctx, tmp_path, shader):
    import xenodon_gb300 as xg
    from xenodon_gb300 import volumes
    g = volumes.blobs(32, seed=4)
    xg.tiff_save(tmp_path / "v.tif", g)
    nodes, st = oracle.build_svo(g, "rope")
    xg.svo_save(tmp_path / "v.svo", nodes, st["side"])
    (tmp_path / "h.conf").write_text("device {\n vkindex = 0\n offset = (0, 0)\n extent = (64, 48)\n}\n")
    _write_cams(tmp_path / "cam.txt")
    vol = "v.tif" if shader == "dda" else "v.svo"
    rc, out = run("render", "--headless", "h.conf", vol, "-s", shader, "--camera", "cam.txt", "-e", "10",
                  "--output", "f-{:0>3}.png", "--stats-output", "stats.txt", "--backend", "cuda", cwd=tmp_path)
    assert rc == 0, out
    assert f"Using shader '{shader}'" in out
    for i, cam in enumerate(CAMS):
        img = png_pixels(tmp_path / f"f-{i:03d}.png")
        ref = oracle.render(shader, grid=g, nodes=nodes, camera=oracle.make_camera(*cam),
                            view=oracle.make_view(64, 48, 10.0))
        assert np.abs(img.astype(int) - ref["rgba"].astype(int)).max() <= 1
    stats = (tmp_path / "stats.txt").read_text().splitlines()
    assert stats[0] == f"total rays: {3 * 64 * 48}"
    assert stats[4] == "frames: 3"
    assert stats[5].startswith("# Frame number: total rays, outputs")
    assert re.fullmatch(r"frame 0: 3072 rays, 1, \S+ ms, \S+ ms, \S+ ms, \S+ mray/s", stats[6])
    assert len(stats) == 9


def test_multi_region_composite_equals_single_region(ctx, tmp_path):
    import xenodon_gb300 as xg
    from xenodon_gb300 import volumes
    g = volumes.blobs(32, seed=6)
    xg.tiff_save(tmp_path / "v.tif", g)
    _write_cams(tmp_path / "cam.txt")
    (tmp_path / "one.conf").write_text("device {\n vkindex = 0\n offset = (0, 0)\n extent = (80, 40)\n}\n")
    (tmp_path / "two.conf").write_text(
        "device {\n vkindex = 0\n offset = (0, 0)\n extent = (30, 40)\n}\n"
        "device {\n vkindex = 1\n offset = (30, 0)\n extent = (50, 40)\n}\n")
    rc, out = run("render", "--headless", "one.conf", "v.tif", "--camera", "cam.txt", "-e", "10", "-q",
                  "--output", "one-{}.png", cwd=tmp_path)
    assert rc == 0, out
    rc, out = run("render", "--headless", "two.conf", "v.tif", "--camera", "cam.txt", "-e", "10",
                  "--output", "two-{}.png", "--repeat", "2", cwd=tmp_path)
    assert rc == 0, out
    assert "Setup: 2 devices, with 1, 1 outputs" in out
    for i in range(3):
        a = png_pixels(tmp_path / f"one-{i}.png")
        b = png_pixels(tmp_path / f"two-{2 * i}.png")
        c = png_pixels(tmp_path / f"two-{2 * i + 1}.png")
        assert np.array_equal(a, b) and np.array_equal(b, c)
    assert not (tmp_path / "two-6.png").exists()


def test_pipelined_frames_equal_serial_frames(ctx, tmp_path):
    """The headless loop queues frame n+1 before it saves frame n (two output
    sets, a saver thread); XN_HEADLESS_SERIAL=1 renders, waits and saves one
    frame at a time.  Both write the same files and the same stats lines, on
    two regions and five frames."""
    import os
    import xenodon_gb300 as xg
    from xenodon_gb300 import cameras, volumes
    g = volumes.blobs(32, seed=7)
    xg.tiff_save(tmp_path / "v.tif", g)
    lines = [" ".join(f"{v:.6f}" for v in (*c[0], *c[1], *c[2]))
             for c in cameras.orbit(np.array([0.5, 0.5, 0.5]), 2.0, 5)]
    (tmp_path / "cam.txt").write_text("\n".join(lines) + "\n")
    (tmp_path / "two.conf").write_text(
        "device {\n vkindex = 0\n offset = (0, 0)\n extent = (40, 30)\n}\n"
        "device {\n vkindex = 1\n offset = (40, 10)\n extent = (24, 30)\n}\n")
    runs = {}
    for mode in ("pipelined", "serial"):
        env = dict(os.environ)
        env.pop("XN_HEADLESS_SERIAL", None)
        if mode == "serial":
            env["XN_HEADLESS_SERIAL"] = "1"
        p = subprocess.run([str(CLI_PATH), "render", "--headless", "two.conf", "v.tif", "--camera", "cam.txt",
                            "-e", "10", "--output", mode + "-{}.png", "--stats-output", mode + ".txt"],
                           capture_output=True, text=True, cwd=tmp_path, timeout=300, env=env)
        assert p.returncode == 0, p.stdout
        runs[mode] = p.stdout
        assert sorted(int(m) for m in re.findall(r"Saved output to '" + mode + r"-(\d+)\.png'", p.stdout)) == \
            list(range(5))
    for i in range(5):
        assert np.array_equal(png_pixels(tmp_path / f"pipelined-{i}.png"), png_pixels(tmp_path / f"serial-{i}.png"))
    a = (tmp_path / "pipelined.txt").read_text().splitlines()
    b = (tmp_path / "serial.txt").read_text().splitlines()
    assert a[0] == b[0] == f"total rays: {5 * (40 * 30 + 24 * 30)}"
    assert [ln.split(":")[0] for ln in a] == [ln.split(":")[0] for ln in b]


def test_camera_script_errors(ctx, tmp_path):
    import xenodon_gb300 as xg
    from xenodon_gb300 import volumes
    xg.tiff_save(tmp_path / "v.tif", volumes.blobs(16, seed=1))
    (tmp_path / "h.conf").write_text("device {\n vkindex = 0\n offset = (0, 0)\n extent = (8, 8)\n}\n")
    (tmp_path / "bad.txt").write_text("0 0 1 0 1 0 0.5 0.5\n")
    rc, out = run("render", "--headless", "h.conf", "v.tif", "--camera", "bad.txt", "-q", "--discard-output",
                  cwd=tmp_path)
    assert rc == 1 and "Error: Syntax error in camera input file" in out
    rc, out = run("render", "--headless", "h.conf", "v.tif", "--camera", "none.txt", "-q", cwd=tmp_path)
    assert rc == 1 and "Error: Failed to open 'none.txt'" in out


@pytest.mark.parametrize("flags,shaders", [(["--rope"], ["svo-rope", "esvo"]), (["--lean"], ["svo-df", "svo-naive"])])
def test_convert_to_device_layout_file_and_render_it(ctx, tmp_path, flags, shaders):
    # .svc destinations hold the device layout; rendering them gives the
    # frames of the same tree converted to .svo
    import xenodon_gb300 as xg
    from xenodon_gb300 import volumes
    g = volumes.blobs(32, seed=9)
    xg.tiff_save(tmp_path / "v.tif", g)
    rc, out = run("convert", *[f for f in flags if f != "--lean"], "v.tif", "v.svo", cwd=tmp_path)
    assert rc == 0, out
    rc, out_svc = run("convert", *flags, "v.tif", "v.svc", cwd=tmp_path)
    assert rc == 0, out_svc
    # the same build report (stats of the same tree)
    assert out.split("Generated octree:")[1] == out_svc.split("Generated octree:")[1]
    (tmp_path / "h.conf").write_text("device {\n vkindex = 0\n offset = (0, 0)\n extent = (40, 30)\n}\n")
    _write_cams(tmp_path / "cam.txt")
    for sh in shaders:
        for vol, pat in (("v.svo", "a-{}.png"), ("v.svc", "b-{}.png")):
            rc, o = run("render", "--headless", "h.conf", vol, "-s", sh, "--camera", "cam.txt", "-e", "10",
                        "--output", pat, cwd=tmp_path)
            assert rc == 0, o
        for i in range(len(CAMS)):
            assert np.array_equal(png_pixels(tmp_path / f"a-{i}.png"), png_pixels(tmp_path / f"b-{i}.png")), sh
