"""The `xenodon` command line: argv, configuration and error behaviour of the
reference's `render` and `convert` (src/main.cpp:97-196, src/convert.cpp:13-122,
src/core/Config.h).  CPU only: every case fails before the GPU is touched."""
from __future__ import annotations

import subprocess

import pytest

from xenodon_gb300 import CLI_PATH


def run(*args, cwd=None):
    p = subprocess.run([str(CLI_PATH), *args], capture_output=True, text=True, cwd=cwd, timeout=60)
    return p.returncode, p.stdout


@pytest.fixture(scope="module")
def conf(tmp_path_factory, built_library):
    d = tmp_path_factory.mktemp("cli")
    (d / "ok.conf").write_text("device {\n    vkindex = 0\n    offset = (0, 0)\n    extent = (64, 48)\n}\n")
    return d


@pytest.mark.parametrize("args,msg", [
    ((), "Missing required positional argument <volume path>"),
    (("v.svo",), "Missing required backend --xorg, --headless or --direct"),
    (("--headless", "ok.conf", "--xorg", "v.svo"), "--xorg, --headless and --direct are mutually exclusive"),
    (("--discard-output", "v.svo", "--xorg"), "--dont-save requires --headless"),
    (("--output", "x.png", "--xorg", "v.svo"), "--output requires --headless"),
    (("--headless", "ok.conf", "--discard-output", "--output", "a.png", "v.svo"),
     "--dont-save and --output are mutually exclusive"),
    (("--headless", "ok.conf", "-e", "-1", "v.svo"), "Invalid value for <emission coefficient> of parameter -e"),
    (("--headless", "ok.conf", "-e", "1e3", "v.svo"), "Invalid value for <emission coefficient> of parameter -e"),
    (("--headless", "ok.conf", "-e", "1", "--emission-coeff", "2", "v.svo"),
     "Duplicate specification of parameter --emission-coeff/-e"),
    (("--headless", "ok.conf", "-q", "-q", "v.svo"), "Duplicate specification of flag --quiet/-q"),
    (("--headless", "ok.conf", "-r", "1:2", "v.svo"), "Invalid value for <voxel dimension ratio> of parameter -r"),
    (("--headless", "ok.conf", "-r", "1:0:2", "v.svo"), "Invalid value for <voxel dimension ratio> of parameter -r"),
    (("--headless", "ok.conf", "--repeat", "0", "v.svo"), "Invalid value for <frame repeat> of parameter --repeat"),
    (("--headless", "ok.conf", "--backend", "vulkan", "v.svo"), "Invalid value for <backend> of parameter --backend"),
    (("--headless", "ok.conf", "v.svo", "w.svo"), "Unexpected positional argument 'w.svo'"),
    (("--headless", "ok.conf", "--bogus", "v.svo"), "Unrecognized option --bogus"),
    (("--headless", "ok.conf", "--camera"), "Parameter --camera expects argument <camera>"),
    (("--headless", "ok.conf", "-q", "v.xyz"), "Failed to parse model file type"),
    (("--headless", "ok.conf", "-q", "-s", "svo-naive", "v.tif"),
     "Shader 'svo-naive' is incompatible with model type 'tiff' (requires 'svo')"),
    (("--headless", "ok.conf", "-q", "-s", "dda", "v.svo"),
     "Shader 'dda' is incompatible with model type 'svo' (requires 'tiff')"),
    (("--headless", "ok.conf", "-q", "-s", "nope", "v.svo"), "Invalid shader 'nope'"),
    (("--headless", "ok.conf", "-q", "--volume-type", "raw", "v.svo"), "Failed to parse model file type"),
])
def test_render_argument_errors(conf, args, msg):
    rc, out = run("render", *args, cwd=conf)
    assert rc == 1
    assert f"Error: {msg}" in out


@pytest.mark.parametrize("text,msg", [
    ("", "Configuration error: At least one device entry is required"),
    ("device {\n vkindex = 0\n offset = (0, 0)\n}\n", "Configuration error: Missing key 'extent'"),
    ("device {\n vkindex = 0\n vkindex = 1\n offset = (0, 0)\n extent = (1, 1)\n}\n",
     "Configuration error: Ambiguous key 'vkindex'"),
    ("device {\n vkindex = 0 # note\n}\n", "Parse error at line 2, col 14: Unexpected character '#'"),
    ("monitor {\n}\n", "Unexpected key 'monitor'"),
    ("device {\n vkindex = x\n}\n", "Expected numeric character, found 'x'"),
    ("device {\n vkindex = 0\n offset = (0 0)\n extent = (1, 1)\n}\n", "Expected character ',', found '0'"),
    ("device {\n vkindex = 0\n offset = (0, 0)\n extent = (1, 1)\n}\n}", "Expected end of input, found '}'"),
])
def test_headless_config_errors(conf, text, msg):
    (conf / "bad.conf").write_text(text)
    rc, out = run("render", "--headless", "bad.conf", "v.svo", cwd=conf)
    assert rc == 1
    assert "Error: Failed to initialize backend: Failed to read config file 'bad.conf': " in out
    assert msg in out


def test_missing_config_file(conf):
    rc, out = run("render", "--headless", "nope.conf", "v.svo", cwd=conf)
    assert "Error: Failed to initialize backend: Failed to open config file 'nope.conf'" in out


@pytest.mark.parametrize("args,msg", [
    (("--dag", "--rope", "a.tif", "b.svo"), "--dag and --rope are mutually exclusive"),
    (("--chan-diff", "3", "--std-dev", "2", "a.tif", "b.svo"), "--std-dev and --chan-diff are mutually exclusive"),
    (("--chan-diff", "256", "a.tif", "b.svo"), "Invalid value for <channel difference> of parameter --chan-diff"),
    (("--std-dev", "-1", "a.tif", "b.svo"), "Invalid value for <std. dev> of parameter --std-dev"),
    (("a.tif",), "Missing required positional argument <destination svo path>"),
    (("--lean", "a.tif", "b.svo"), "--lean builds a sparse tree into a .svc file (no --dag or --rope)"),
    (("--lean", "--rope", "a.tif", "b.svc"), "--lean builds a sparse tree into a .svc file (no --dag or --rope)"),
])
def test_convert_argument_errors(conf, args, msg):
    rc, out = run("convert", *args, cwd=conf)
    assert rc == 1 and f"Error: {msg}" in out


def test_convert_missing_source(conf):
    rc, out = run("convert", "nope.tif", "out.svo", cwd=conf)
    assert out.startswith("Loading source...\n")
    assert "Error reading 'nope.tif': Failed to open" in out


def test_help_and_unknown_subcommand(built_library):
    rc, out = run()
    assert rc == 0 and "render" in out and "convert" in out
    rc, out = run("help", "render")
    assert rc == 0 and "--headless" in out
    rc, out = run("help", "nope")
    assert rc == 1 and "Error: No such topic nope" in out
    rc, out = run("bogus")
    assert rc == 1 and "Error: Invalid subcommand 'bogus'" in out


_CONF_DRIVER = r'''
#include <cstdio>
#include <fstream>
#include <sstream>
#include "cli_util.h"
// prints what the command line's headless.conf parser makes of a file, in the
// form of oracle/ref_config_driver.cpp
int main(int argc, char** argv) {
    std::ifstream in(argv[1], std::ios::binary);
    std::stringstream ss;
    ss << in.rdbuf();
    try {
        for (const auto& d : cli::parse_headless_config(ss.str()))
            std::printf("device %u %d %d %u %u\n", (unsigned)d.vkindex, d.region.x, d.region.y, d.region.width,
                        d.region.height);
    } catch (const cli::Error& e) {
        std::string m = e.what();
        std::printf("error: ");
        std::fwrite(m.data(), 1, m.size(), stdout);
        std::printf("\n");
    }
    return 0;
}
'''


def test_headless_conf_parser_matches_the_reference(tmp_path):
    # the reference's own parser (src/core/Parser.cpp, Config.h,
    # src/backend/headless/HeadlessConfig.cpp, compiled by `make -C oracle
    # ref-config`) and the command line's, on edge cases and 1500 random
    # mutations of valid files: the same devices, or the same error message
    import random
    from pathlib import Path
    import oracle
    if not oracle.build_ref_config():
        pytest.skip("reference sources not present")
    root = Path(__file__).resolve().parents[1]
    drv = tmp_path / "conf.cpp"
    drv.write_text(_CONF_DRIVER)
    ours = tmp_path / "conf"
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", str(root / "xenodon_gb300" / "host"), "-I",
                    str(root / "include"), str(drv), str(root / "xenodon_gb300" / "host" / "cli_util.cpp"), "-o",
                    str(ours)], check=True)
    valid = [
        "device {\n  vkindex = 0\n  offset = (0, 0)\n  extent = (512, 512)\n}\n",
        "device { vkindex = 0 offset = (0, 0) extent = (960, 1080) }\n"
        "device { vkindex = 1 offset = (960, 0) extent = (960, 1080) }\n",
        "# a comment\ndevice {\n\tvkindex = 3\n\textent = (17, 4)\n\toffset = (5, 6)\n}\n# trailing\n",
        "device{vkindex=0 offset=(1,2) extent=(3,4)}",
        "device {\n  vkindex = 0\n  offset = ( 0 , 0 )\n  extent = ( 512 , 512 )\n}\n\n\n",
    ]
    cases = valid + [
        "", "\n", "device {}", "device { vkindex = 0 }", "Device { }", "8device{}",
        "device { vkindex = 99999999999999999999 offset = (4294967296, 2147483648) extent = (4294967297, 0) }",
        "device { vkindex = 0 offset = (0, 0) extent = (1, 1) } x",
        "device { vkindex = 0 vkindex = 1 offset = (0,0) extent=(1,1) }",
        "device { vkindex = 0 offset = (0, 0) extent = (1, 1) }#c",
        "device { vkindex = 0 offset = (0, 0) extent = (1, 1) \n",
        "device\n{ vkindex = 0 offset = (0,0) extent=(1,1) }",
        "device { vkindex = 0\n offset = (0, 0)\nvkindex  extent = (1, 1) }",
    ]
    alphabet = list("{}()=,#\n \t\r0123456789abcdevkinxofsetrzq\"\\-+") + ["device", "vkindex", "offset", "extent"]
    rng = random.Random(5)
    for _ in range(1500):
        s = list(rng.choice(valid))
        for _ in range(rng.randint(1, 6)):
            i = rng.randint(0, len(s))
            op = rng.random()
            if op < 0.35 and s:
                del s[min(i, len(s) - 1)]
            elif op < 0.7:
                s.insert(i, rng.choice(alphabet))
            elif s:
                s[min(i, len(s) - 1)] = rng.choice(alphabet)
        cases.append("".join(s))
    f = tmp_path / "c.conf"
    for c in cases:
        f.write_bytes(c.encode())
        ref = subprocess.run([str(oracle.REF_CONFIG), str(f)], capture_output=True, timeout=30).stdout
        got = subprocess.run([str(ours), str(f)], capture_output=True, timeout=30).stdout
        assert got == ref, (c, ref, got)


_RECT_DRIVER = r'''
#include <cstdio>
#include <iostream>
#include <vector>
#include "cli_util.h"
// the command line's rect_union, in the form of oracle/ref_rect_driver.cpp
int main() {
    size_t n;
    while (std::cin >> n) {
        std::vector<cli::Rect> rects(n);
        for (auto& r : rects) std::cin >> r.x >> r.y >> r.width >> r.height;
        cli::Rect pair = n >= 2 ? cli::rect_union(rects[0], rects[1]) : cli::Rect{};
        cli::Rect all = cli::rect_union_composite(rects);
        std::printf("%d %d %u %u | %d %d %u %u\n", pair.x, pair.y, pair.width, pair.height, all.x, all.y, all.width,
                    all.height);
    }
    return 0;
}
'''


def test_rect_union_matches_the_reference(tmp_path):
    # the reference's rect_union (src/utility/rect_union.h: the two-rectangle
    # form and the iterator form the saved composite uses, which takes its y
    # origin from x) against the command line's, on 3000 random lists of 0 to
    # 6 rectangles, negative offsets and sizes near the 32-bit limits included
    import random
    from pathlib import Path
    import oracle
    if not oracle.build_ref_rect():
        pytest.skip("reference sources not present")
    root = Path(__file__).resolve().parents[1]
    drv = tmp_path / "rect.cpp"
    drv.write_text(_RECT_DRIVER)
    ours = tmp_path / "rect"
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", str(root / "xenodon_gb300" / "host"), "-I",
                    str(root / "include"), str(drv), str(root / "xenodon_gb300" / "host" / "cli_util.cpp"), "-o",
                    str(ours)], check=True)
    rng = random.Random(9)
    lines = []
    for _ in range(3000):
        n = rng.randint(0, 6)
        vals = [n]
        for _ in range(n):
            big = rng.random() < 0.1
            vals += [rng.randint(-2**31, 2**31 - 1) if big else rng.randint(-2000, 4000),
                     rng.randint(-2**31, 2**31 - 1) if big else rng.randint(-2000, 4000),
                     rng.randint(0, 2**32 - 1) if big else rng.randint(0, 4000),
                     rng.randint(0, 2**32 - 1) if big else rng.randint(0, 4000)]
        lines.append(" ".join(map(str, vals)))
    text = "\n".join(lines) + "\n"
    ref = subprocess.run([str(oracle.REF_RECT)], input=text, capture_output=True, text=True, timeout=60).stdout
    got = subprocess.run([str(ours)], input=text, capture_output=True, text=True, timeout=60).stdout
    for line, a, b in zip(lines, ref.splitlines(), got.splitlines()):
        assert a == b, (line, a, b)
    assert len(ref.splitlines()) == len(lines) == len(got.splitlines())
