"""Host file formats through the C ABI (CPU only): stacked TIFF as
TIFFReadRGBAImage hands it to the reference (src/model/Grid.cpp:27-79) and
PNG frames."""
from __future__ import annotations

import struct
import zlib

import numpy as np
import pytest


def _lzw_encode(data: bytes) -> bytes:
    """TIFF LZW, MSB-first: codes are written at the width the decoder reads
    them with, which grows when its next free entry reaches 2^width - 1."""
    def width(dec_next):
        return 12 if dec_next >= 2047 else 11 if dec_next >= 1023 else 10 if dec_next >= 511 else 9

    codes = []
    table = {bytes([i]): i for i in range(256)}
    next_code, dec_next, first = 258, 258, True
    codes.append((256, 9))
    w = b""
    for c in data:
        wc = w + bytes([c])
        if wc in table:
            w = wc
            continue
        codes.append((table[w], width(dec_next)))
        if first:
            first = False
        else:
            dec_next += 1
        table[wc] = next_code
        next_code += 1
        w = bytes([c])
        if next_code >= 4093:  # table full: clear, both sides start over
            codes.append((256, width(dec_next)))
            table = {bytes([i]): i for i in range(256)}
            next_code, dec_next, first = 258, 258, True
    if w:
        codes.append((table[w], width(dec_next)))
        if not first:
            dec_next += 1
    codes.append((257, width(dec_next)))
    bits = "".join(format(c, f"0{n}b") for c, n in codes)
    bits += "0" * (-len(bits) % 8)
    return int(bits, 2).to_bytes(len(bits) // 8, "big") if bits else b""


def _packbits_encode(data: bytes) -> bytes:
    out = bytearray()
    i = 0
    while i < len(data):
        run = 1
        while i + run < len(data) and run < 128 and data[i + run] == data[i]:
            run += 1
        if run >= 3:
            out += bytes([(257 - run) & 0xFF, data[i]])
            i += run
            continue
        j = i
        while j < len(data) and j - i < 128 and not (j + 2 < len(data) and data[j] == data[j + 1] == data[j + 2]):
            j += 1
        out += bytes([j - i - 1]) + data[i:j]
        i = j
    return bytes(out)


def _encode_chunk(raw: bytes, compression: int, predictor: int, row_bytes: int, spp: int) -> bytes:
    if predictor == 2:
        a = np.frombuffer(raw, np.uint8).reshape(-1, row_bytes).astype(np.int32)
        d = a.copy()
        d[:, spp:] = a[:, spp:] - a[:, :-spp]
        raw = (d & 0xFF).astype(np.uint8).tobytes()
    if compression == 1:
        return raw
    if compression in (8, 32946):
        return zlib.compress(raw, 6)
    if compression == 5:
        return _lzw_encode(raw)
    if compression == 32773:
        return _packbits_encode(raw)
    raise ValueError(compression)


def _classic_tiff(pages, photometric, spp, extra=None, big_endian=False, tile=None, compression=1, predictor=1,
                  rows_per_strip=None):
    """Minimal independent TIFF writer: pages is a list of uint8 (h, w, spp)."""
    e = ">" if big_endian else "<"
    out = bytearray(b"MM" if big_endian else b"II")
    out += struct.pack(e + "HI", 42, 8)
    offsets = []
    for i, img in enumerate(pages):
        h, w = img.shape[:2]
        entries = []
        data_parts = []
        if tile:
            tw, th = tile
            tx, ty = -(-w // tw), -(-h // th)
            for j in range(ty):
                for k in range(tx):
                    t = np.zeros((th, tw, spp), np.uint8)
                    blk = img[j * th:(j + 1) * th, k * tw:(k + 1) * tw]
                    t[:blk.shape[0], :blk.shape[1]] = blk
                    data_parts.append(_encode_chunk(t.tobytes(), compression, predictor, tw * spp, spp))
        else:
            rps = rows_per_strip or h
            for y in range(0, h, rps):
                data_parts.append(_encode_chunk(img[y:y + rps].tobytes(), compression, predictor, w * spp, spp))
        n_entries = 10 + (1 if extra is not None else 0) + (1 if tile else 0) + (1 if predictor != 1 else 0)
        ifd_off = len(out)
        after_ifd = ifd_off + 2 + 12 * n_entries + 4
        bps_off = after_ifd
        offs_off = bps_off + 2 * spp
        cnt_off = offs_off + 4 * len(data_parts)
        data_off = cnt_off + 4 * len(data_parts)
        poffs, pcnts = [], []
        p = data_off
        for d in data_parts:
            poffs.append(p)
            pcnts.append(len(d))
            p += len(d)
        next_off = p if i + 1 < len(pages) else 0

        def ent(tag, typ, count, value):
            if typ == 3 and count == 1:
                return struct.pack(e + "HHIHH", tag, typ, count, value, 0)
            return struct.pack(e + "HHII", tag, typ, count, value)

        entries.append(ent(256, 4, 1, w))
        entries.append(ent(257, 4, 1, h))
        entries.append(ent(258, 3, spp, bps_off) if spp > 2 else ent(258, 3, 1, 8))
        entries.append(ent(259, 3, 1, compression))
        entries.append(ent(262, 3, 1, photometric))
        entries.append(ent(324 if tile else 273, 4, len(poffs), offs_off if len(poffs) > 1 else poffs[0]))
        entries.append(ent(277, 3, 1, spp))
        if tile:
            entries.append(ent(322, 3, 1, tile[0]))
            entries.append(ent(323, 3, 1, tile[1]))
        else:
            entries.append(ent(278, 4, 1, rows_per_strip or h))
        entries.append(ent(325 if tile else 279, 4, len(pcnts), cnt_off if len(pcnts) > 1 else pcnts[0]))
        entries.append(ent(284, 3, 1, 1))
        if extra is not None:
            entries.append(ent(338, 3, 1, extra))
        if predictor != 1:
            entries.append(ent(317, 3, 1, predictor))
        entries.sort(key=lambda b: struct.unpack(e + "H", b[:2])[0])
        assert len(entries) == n_entries
        out += struct.pack(e + "H", n_entries) + b"".join(entries) + struct.pack(e + "I", next_off)
        out += struct.pack(e + "H" * spp, *([8] * spp))
        out += struct.pack(e + "I" * len(poffs), *poffs)
        out += struct.pack(e + "I" * len(pcnts), *pcnts)
        for d in data_parts:
            out += d
        offsets.append(ifd_off)
    return bytes(out)


def test_tiff_gray_pages_are_bottom_up_rgb(built_library, tmp_path):
    import xenodon_gb300 as xg
    rng = np.random.default_rng(0)
    pages = [rng.integers(0, 256, (5, 7, 1)).astype(np.uint8) for _ in range(3)]
    p = tmp_path / "g.tif"
    p.write_bytes(_classic_tiff(pages, photometric=1, spp=1))
    g = xg.tiff_load(p)
    assert g.shape == (3, 5, 7, 4)
    for z, img in enumerate(pages):
        for y in range(5):
            assert np.array_equal(g[z, y, :, 0], img[4 - y, :, 0])  # grid row y = image row h-1-y
    assert np.array_equal(g[..., 0], g[..., 1]) and np.array_equal(g[..., 0], g[..., 2])
    assert np.all(g[..., 3] == 255)


@pytest.mark.parametrize("big_endian", [False, True])
def test_tiff_rgb_and_tiles(built_library, tmp_path, big_endian):
    import xenodon_gb300 as xg
    rng = np.random.default_rng(1)
    pages = [rng.integers(0, 256, (9, 11, 3)).astype(np.uint8) for _ in range(2)]
    for tile in (None, (16, 16)):
        p = tmp_path / "rgb.tif"
        p.write_bytes(_classic_tiff(pages, photometric=2, spp=3, big_endian=big_endian, tile=tile))
        g = xg.tiff_load(p)
        assert g.shape == (2, 9, 11, 4)
        for z in range(2):
            assert np.array_equal(g[z, :, :, :3], pages[z][::-1])
        assert np.all(g[..., 3] == 255)


def test_tiff_rgba_alpha_handling(built_library, tmp_path):
    import xenodon_gb300 as xg
    rng = np.random.default_rng(2)
    img = rng.integers(0, 256, (4, 6, 4)).astype(np.uint8)
    # associated alpha: kept as stored
    p = tmp_path / "a.tif"
    p.write_bytes(_classic_tiff([img], photometric=2, spp=4, extra=1))
    assert np.array_equal(xg.tiff_load(p)[0], img[::-1])
    # unassociated alpha: premultiplied as libtiff's RGBA interface does
    p.write_bytes(_classic_tiff([img], photometric=2, spp=4, extra=2))
    got = xg.tiff_load(p)[0]
    a = img[..., 3:4].astype(np.uint32)
    exp = img.copy()
    exp[..., :3] = ((img[..., :3].astype(np.uint32) * a + 127) // 255).astype(np.uint8)
    assert np.array_equal(got, exp[::-1])


def test_tiff_roundtrip_of_own_writer(built_library, tmp_path):
    import xenodon_gb300 as xg
    from xenodon_gb300 import volumes
    g = volumes.random_grid(6, 5, 9, seed=3)  # alpha 255: unchanged by premultiplication
    xg.tiff_save(tmp_path / "v.tif", g)
    assert np.array_equal(xg.tiff_load(tmp_path / "v.tif"), g)


@pytest.mark.parametrize("data,msg", [
    (b"XX*\x00" + b"\0" * 20, "not a TIFF"),
    (b"II*\x00\x08\x00\x00\x00\x05", "truncated directory"),
])
def test_tiff_malformed(built_library, tmp_path, data, msg):
    import xenodon_gb300 as xg
    p = tmp_path / "bad.tif"
    p.write_bytes(data)
    with pytest.raises(xg.XenodonError) as e:
        xg.tiff_load(p)
    assert msg in str(e.value)


def test_tiff_missing_file(built_library, tmp_path):
    import xenodon_gb300 as xg
    with pytest.raises(xg.XenodonError) as e:
        xg.tiff_load(tmp_path / "nope.tif")
    assert "Failed to open" in str(e.value)


def test_tiff_layer_size_check_follows_reference(built_library, tmp_path):
    # Grid.cpp:47 rejects a layer only when width AND height differ
    import xenodon_gb300 as xg
    a = np.zeros((4, 5, 1), np.uint8)
    b = np.zeros((3, 6, 1), np.uint8)
    p = tmp_path / "d.tif"
    p.write_bytes(_classic_tiff([a, b], photometric=1, spp=1))
    with pytest.raises(xg.XenodonError) as e:
        xg.tiff_load(p)
    assert "differ from previous dimensions" in str(e.value)
    c = np.zeros((4, 6, 1), np.uint8)  # same height: accepted like the reference
    p.write_bytes(_classic_tiff([a, c], photometric=1, spp=1))
    assert xg.tiff_load(p).shape == (2, 4, 5, 4)


def _png_decode(data: bytes) -> np.ndarray:
    from pngdec import decode
    return decode(data)


@pytest.mark.parametrize("shape", [(1, 1), (33, 47), (300, 251)])
def test_png_decodes_to_the_pixels(built_library, tmp_path, shape):
    import xenodon_gb300 as xg
    img = np.random.default_rng(4).integers(0, 256, shape + (4,)).astype(np.uint8)
    xg.png_save(tmp_path / "f.png", img)
    assert np.array_equal(_png_decode((tmp_path / "f.png").read_bytes()), img)


def test_png_compresses_a_rendered_frame(built_library, tmp_path):
    """A frame-like image (black background, opaque alpha, a smooth disc and
    noise) round-trips through zlib and compresses well below its raw size;
    its rows span several parallel deflate bands."""
    import xenodon_gb300 as xg
    h, w = 720, 1280
    yy, xx = np.mgrid[0:h, 0:w]
    r = np.hypot(yy - h / 2, xx - w / 2)
    img = np.zeros((h, w, 4), np.uint8)
    img[..., 3] = 255
    disc = r < 250
    img[..., 0] = np.where(disc, (255 - r).clip(0, 255), 0).astype(np.uint8)
    img[..., 1] = np.where(disc, (xx % 256), 0).astype(np.uint8)
    rng = np.random.default_rng(1)
    img[300:340, 100:400, 2] = rng.integers(0, 256, (40, 300))
    xg.png_save(tmp_path / "f.png", img)
    data = (tmp_path / "f.png").read_bytes()
    assert np.array_equal(_png_decode(data), img)
    assert len(data) < img.nbytes / 8
    blank = np.zeros((64, 4000, 4), np.uint8)
    xg.png_save(tmp_path / "b.png", blank)
    assert np.array_equal(_png_decode((tmp_path / "b.png").read_bytes()), blank)


def test_png_files_decode_with_the_reference_png_library(built_library, tmp_path):
    # the PNG library the reference writes its frames with (subprojects/lodepng,
    # compiled by `make -C oracle ref-png`) decodes the library's PNG files,
    # every filter and deflate path among them, to exactly their pixels
    import subprocess
    import oracle
    import xenodon_gb300 as xg
    if not oracle.build_ref_png():
        pytest.skip("reference sources not present")
    rng = np.random.default_rng(11)
    h, w = 720, 1280
    yy, xx = np.mgrid[0:h, 0:w]
    r = np.hypot(yy - h / 2, xx - w / 2)
    frame = np.zeros((h, w, 4), np.uint8)
    frame[..., 3] = 255
    frame[..., 0] = np.where(r < 250, (255 - r).clip(0, 255), 0).astype(np.uint8)
    frame[..., 1] = np.where(r < 250, xx % 256, 0).astype(np.uint8)
    frame[300:340, 100:400, 2] = rng.integers(0, 256, (40, 300))
    images = [rng.integers(0, 256, s + (4,)).astype(np.uint8) for s in ((1, 1), (3, 7), (33, 47), (2, 1920))]
    images += [frame, np.zeros((64, 4000, 4), np.uint8), np.full((17, 5, 4), 255, np.uint8)]
    for k, img in enumerate(images):
        f, raw = tmp_path / f"{k}.png", tmp_path / f"{k}.rgba"
        xg.png_save(f, img)
        out = subprocess.run([str(oracle.REF_PNG), str(f), str(raw)], capture_output=True, text=True,
                             timeout=60).stdout
        assert out.strip() == f"ok {img.shape[1]} {img.shape[0]}", out
        assert np.array_equal(np.fromfile(raw, np.uint8).reshape(img.shape), img), k


@pytest.mark.parametrize("compression", [5, 8, 32946, 32773])
@pytest.mark.parametrize("predictor", [1, 2])
@pytest.mark.parametrize("layout", ["strips", "tiles"])
def test_tiff_compressed_pages_equal_uncompressed(built_library, tmp_path, compression, predictor, layout):
    # LZW, Deflate and PackBits (+ the horizontal predictor), as libtiff
    # decodes them for TIFFReadRGBAImage
    import xenodon_gb300 as xg
    rng = np.random.default_rng(7)
    yy, xx = np.mgrid[0:37, 0:29]
    pages = []
    for z in range(3):
        img = np.stack([(xx * 7 + z) % 256, (yy * 3) % 256, rng.integers(0, 4, (37, 29)) * 60], -1)
        img[10:20] = 0  # runs
        pages.append(img.astype(np.uint8))
    kw = {"tile": (16, 16)} if layout == "tiles" else {"rows_per_strip": 5}
    p = tmp_path / "c.tif"
    p.write_bytes(_classic_tiff(pages, photometric=2, spp=3, compression=compression, predictor=predictor, **kw))
    q = tmp_path / "u.tif"
    q.write_bytes(_classic_tiff(pages, photometric=2, spp=3))
    assert np.array_equal(xg.tiff_load(p), xg.tiff_load(q))


def test_tiff_lzw_long_page_grows_the_code_width_and_clears(built_library, tmp_path):
    # 64 KiB of noise: every code width 9..12 and at least one Clear code
    import xenodon_gb300 as xg
    rng = np.random.default_rng(8)
    img = rng.integers(0, 256, (128, 128, 4)).astype(np.uint8)
    p = tmp_path / "l.tif"
    p.write_bytes(_classic_tiff([img], photometric=2, spp=4, extra=1, compression=5))
    assert np.array_equal(xg.tiff_load(p)[0], img[::-1])


@pytest.mark.parametrize("compression", [5, 8, 32773])
def test_tiff_corrupt_compressed_strip_is_an_error(built_library, tmp_path, compression):
    import xenodon_gb300 as xg
    img = np.arange(8 * 8 * 3, dtype=np.uint8).reshape(8, 8, 3)
    data = bytearray(_classic_tiff([img], photometric=2, spp=3, compression=compression))
    good = _encode_chunk(img.tobytes(), compression, 1, 24, 3)
    at = bytes(data).index(good)
    data[at:at + len(good)] = good[: len(good) // 2] + bytes(len(good) - len(good) // 2)  # zeroed second half
    p = tmp_path / "x.tif"
    p.write_bytes(bytes(data))
    with pytest.raises(xg.XenodonError) as e:
        xg.tiff_load(p)
    assert "corrupt compressed strip" in str(e.value)


def test_tiff_unknown_compression_is_an_error(built_library, tmp_path):
    import xenodon_gb300 as xg
    img = np.zeros((4, 4, 3), np.uint8)
    data = _classic_tiff([img], photometric=2, spp=3)
    entry = struct.pack("<HHIHH", 259, 3, 1, 1, 0)
    data = data.replace(entry, struct.pack("<HHIHH", 259, 3, 1, 7, 0))  # JPEG
    p = tmp_path / "j.tif"
    p.write_bytes(data)
    with pytest.raises(xg.XenodonError) as e:
        xg.tiff_load(p)
    assert "compression 7 is not supported" in str(e.value)
