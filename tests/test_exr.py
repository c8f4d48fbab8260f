"""EXR output (vg_write_exr) and the exr_diff gates, on the CPU. The writer cases restate the
reference's tests in crates/verion-render-io/src/exr_out.rs:341-549; the reader is checked on files
this writer makes and on RLE / ZIP encodings made here from the OpenEXR layout."""
import struct
import zlib

import numpy as np
import pytest

from verion_gb300 import exr
from verion_gb300.backend import Error
from verion_gb300.exr_diff import main as exr_diff_main


def info(**kw):
    base = dict(physical=True, samples=64, stylization_revision=3)
    base.update(kw)
    return exr.RenderInfo(**base)


def test_writes_beauty_normal_and_metadata(tmp_path):
    p = tmp_path / "aov.exr"
    exr.write_exr(p, 2, 1, [[1.0, 2.0, 3.0], [0.25, 0.5, 4.0]], normal=[[0.0, 0.0, 1.0], [1.0, 0.0, 0.0]], info=info())
    img = exr.read_exr(p)
    assert list(img.channels["R"][0]) == [1.0, 0.25]
    assert list(img.channels["B"][0]) == [3.0, 4.0]
    assert list(img.channels["N.Z"][0]) == [1.0, 0.0]
    a = img.attributes
    assert a["verion/physical"] == "true"
    assert a["verion/samples"] == 64
    assert a["verion/stylizationRevision"] == "3"
    assert a["chromaticities"][:2] == pytest.approx((0.64, 0.33))
    assert a["verion/workingSpace"] == "LinearRec709"
    assert a["verion/outputTransform"] == "OutputTransform { target: LinearRec709, tone_map: None, oetf: Linear }"


def test_records_the_color_grade_only_when_one_was_applied(tmp_path):
    beauty = np.zeros((2, 3))

    def attrs(i):
        p = tmp_path / "g.exr"
        exr.write_exr(p, 2, 1, beauty, info=i)
        return exr.read_exr(p).attributes

    plain = attrs(info())
    assert "verion/exposure" not in plain and "verion/denoiser" not in plain
    d = attrs(info(denoiser="oidn"))
    assert d["verion/denoiser"] == "oidn" and d["verion/physical"] == "false"
    d = attrs(info(adaptive_threshold=0.02))
    assert d["verion/adaptiveThreshold"] == np.float32(0.02) and d["verion/physical"] == "false"
    d = attrs(info(restir="di+gi"))
    assert d["verion/restir"] == "di+gi" and d["verion/physical"] == "false"
    d = attrs(info(grade=(-1.0, 0.8, (1.1, 1.0, 0.9))))
    assert d["verion/exposure"] == -1.0 and d["verion/saturation"] == np.float32(0.8)
    assert d["verion/whiteBalance"] == tuple(np.float32(x) for x in (1.1, 1.0, 0.9))


def test_writes_albedo_depth_and_object_id(tmp_path):
    p = tmp_path / "ids.exr"
    kw = dict(albedo=[[1.0, 0.0, 0.0], [0.5, 0.5, 0.5]], depth=[3.0, 0.0], object_id=[7, 0], material_id=[3, 0],
              sample_count=[16, 64])
    exr.write_exr(p, 2, 1, np.zeros((2, 3)), info=info(), **kw)
    img = exr.read_exr(p)
    assert list(img.channels["Albedo.R"][0]) == [1.0, 0.5]
    assert list(img.channels["Z"][0]) == [3.0, 0.0]
    assert list(img.channels["ObjectId"][0]) == [7, 0] and img.channels["ObjectId"].dtype == np.uint32
    assert list(img.channels["MaterialId"][0]) == [3, 0]
    assert list(img.channels["SampleCount"][0]) == [16, 64]
    kw["depth"] = [1.0]
    with pytest.raises(Error):
        exr.write_exr(p, 2, 1, np.zeros((2, 3)), info=info(), **kw)


def test_converts_primaries_and_marks_display_output_non_physical(tmp_path):
    p = tmp_path / "aces.exr"
    beauty = [[1.0, 0.0, 0.0], [0.0, 0.0, 0.0]]
    exr.write_exr(p, 2, 1, beauty, info=info(), target=exr.COLOR_ACESCG)
    img = exr.read_exr(p)
    assert abs(img.channels["R"][0, 0] - 0.613097) < 1e-6
    assert img.attributes["chromaticities"][6:] == pytest.approx((0.32168, 0.33767))
    # load_hdri converts an ACEScg file back to Rec.709.
    assert np.allclose(exr.beauty_rec709(img)[0], [1.0, 0.0, 0.0], atol=1e-4)
    exr.write_exr(p, 2, 1, beauty, info=info(), tone_map=exr.TONEMAP_REINHARD, oetf=exr.OETF_SRGB)
    img = exr.read_exr(p)
    assert img.attributes["verion/physical"] == "false"
    # color.rs:186-196: Reinhard maps luminance 1 to 0.5; sRGB encodes 0.5 as about 0.7354.
    exr.write_exr(p, 1, 1, [[1.0, 1.0, 1.0]], info=info(), tone_map=exr.TONEMAP_REINHARD, oetf=exr.OETF_SRGB)
    assert abs(exr.read_exr(p).channels["G"][0, 0] - 0.7354) < 1e-3


def test_rejects_mismatched_frames(tmp_path):
    p = tmp_path / "bad.exr"
    with pytest.raises(Error):
        exr.write_exr(p, 2, 1, [[0.0, 0.0, 0.0]], info=info())
    with pytest.raises(Error):
        exr.write_exr(p, 2, 1, np.zeros((2, 3)), normal=[[0.0, 0.0, 0.0]], info=info())
    with pytest.raises(Error):
        exr.write_exr(p, 0, 0, np.zeros((0, 3)), info=info())


def test_writes_lighting_parts(tmp_path):
    p = tmp_path / "lighting.exr"

    def part(v):
        return [[v, 2 * v, 3 * v]] * 2

    parts = [part(1.0), part(2.0), part(3.0), part(4.0), part(5.0)]
    exr.write_exr(p, 2, 1, np.zeros((2, 3)), lighting=parts, visibility=[0.25, 1.0], info=info())
    c = exr.read_exr(p).channels
    assert list(c["DirectDiffuse.G"][0]) == [2.0, 2.0]
    assert list(c["IndirectDiffuse.R"][0]) == [2.0, 2.0]
    assert list(c["Specular.B"][0]) == [9.0, 9.0]
    assert list(c["Transmission.R"][0]) == [4.0, 4.0]
    assert list(c["Emission.R"][0]) == [5.0, 5.0]
    assert list(c["Visibility.V"][0]) == [0.25, 1.0]
    with pytest.raises(Error):
        exr.write_exr(p, 2, 1, np.zeros((2, 3)), lighting=parts, visibility=[1.0], info=info())


# ---- reader on compressed files ------------------------------------------------------------------

def _predict_and_interleave(raw: bytes) -> bytes:
    a = np.frombuffer(raw, np.uint8)
    t = np.concatenate([a[0::2], a[1::2]]).astype(np.int64)
    d = t.copy()
    d[1:] = (t[1:] - t[:-1] + 128 + 256) & 0xFF
    return d.astype(np.uint8).tobytes()


def _rle_encode(b: bytes) -> bytes:
    out = bytearray()
    i = 0
    while i < len(b):
        j = i
        while j < len(b) and j - i < 127 and b[j] == b[i]:
            j += 1
        if j - i >= 3:
            out += struct.pack("b", j - i - 1) + b[i:i + 1]
            i = j
        else:
            k = i
            while k < len(b) and k - i < 127 and not (k + 2 < len(b) and b[k] == b[k + 1] == b[k + 2]):
                k += 1
            k = max(k, i + 1)
            out += struct.pack("b", -(k - i)) + b[i:k]
            i = k
    return bytes(out)


def _write_compressed(path, comp, w, h, planes):
    """A FLOAT-channel scanline file with RLE (1) or ZIP (3) chunks, channels in name order."""
    names = sorted(planes)
    hdr = bytearray(struct.pack("<II", 20000630, 2))

    def attr(name, typ, val):
        hdr.extend(name.encode() + b"\0" + typ.encode() + b"\0" + struct.pack("<i", len(val)) + val)

    ch = b"".join(n.encode() + b"\0" + struct.pack("<iB3sii", 2, 0, b"\0\0\0", 1, 1) for n in names) + b"\0"
    attr("channels", "chlist", ch)
    attr("compression", "compression", bytes([comp]))
    attr("dataWindow", "box2i", struct.pack("<4i", 0, 0, w - 1, h - 1))
    attr("displayWindow", "box2i", struct.pack("<4i", 0, 0, w - 1, h - 1))
    attr("lineOrder", "lineOrder", b"\0")
    attr("pixelAspectRatio", "float", struct.pack("<f", 1.0))
    attr("screenWindowCenter", "v2f", struct.pack("<2f", 0, 0))
    attr("screenWindowWidth", "float", struct.pack("<f", 1.0))
    hdr += b"\0"
    lines = 16 if comp == 3 else 1
    chunks = []
    for y in range(0, h, lines):
        raw = b"".join(np.asarray(planes[n][yy], "<f4").tobytes() for yy in range(y, min(h, y + lines)) for n in names)
        pre = _predict_and_interleave(raw)
        data = zlib.compress(pre) if comp == 3 else _rle_encode(pre)
        if len(data) >= len(raw):
            data = raw
        chunks.append(struct.pack("<ii", y, len(data)) + data)
    off = len(hdr) + 8 * len(chunks)
    table = b""
    for c in chunks:
        table += struct.pack("<Q", off)
        off += len(c)
    open(path, "wb").write(bytes(hdr) + table + b"".join(chunks))


@pytest.mark.parametrize("comp", [1, 3])
def test_reader_decodes_rle_and_zip(tmp_path, comp):
    w, h = 37, 21
    rng = np.random.default_rng(comp)
    y, x = np.mgrid[0:h, 0:w]
    planes = {"R": (x / w).astype(np.float32), "G": np.full((h, w), 0.5, np.float32),
              "B": rng.uniform(0, 4, (h, w)).astype(np.float32)}
    p = tmp_path / "c.exr"
    _write_compressed(p, comp, w, h, planes)
    img = exr.read_exr(p)
    for n in planes:
        assert np.array_equal(img.channels[n], planes[n]), n


# ---- exr_diff ------------------------------------------------------------------------------------

def _img(w=64, h=48, seed=0):
    rng = np.random.default_rng(seed)
    return rng.uniform(0.2, 1.0, (h * w, 3)).astype(np.float32)


def test_diff_gates():
    w, h = 64, 48
    r = _img()
    d = exr.diff(r, r, w, h)
    assert d["channel"] == 0.0 and d["block"] == 0.0 and d["pass"] and d["psnr_db"] == float("inf")
    assert exr.diff(r, r * 1.005, w, h)["pass"]
    d = exr.diff(r, r * 1.015, w, h)
    assert not d["pass"] and d["channel"] == pytest.approx(0.015, rel=1e-6)
    # One 4x4 block brighter by 3%: channel means move by ~0.2%, the block gate fails.
    t = r.reshape(h, w, 3).copy()
    t[:h // 4, :w // 4] *= 1.03
    d = exr.diff(r, t.reshape(-1, 3), w, h)
    assert d["channel"] < 0.01 and d["block"] == pytest.approx(0.03, rel=1e-5) and not d["pass"]


def test_exr_diff_command(tmp_path, capsys, monkeypatch):
    w, h = 32, 16
    r = _img(w, h, 1)
    ref, same, off = tmp_path / "ref.exr", tmp_path / "same.exr", tmp_path / "off.exr"
    exr.write_exr(ref, w, h, r, info=info())
    exr.write_exr(same, w, h, r * 1.004, info=info())
    exr.write_exr(off, w, h, r * 1.02, info=info())
    assert exr_diff_main([str(ref), str(same)]) == 0
    assert "PASS" in capsys.readouterr().out
    assert exr_diff_main([str(ref), str(same), str(off)]) == 1
    out = capsys.readouterr().out
    assert out.count("PASS") == 1 and out.count("FAIL") == 1
    monkeypatch.setenv("EXR_DIFF_CHANNEL", "0.05")
    monkeypatch.setenv("EXR_DIFF_BLOCK", "0.05")
    assert exr_diff_main([str(ref), str(off)]) == 0
    assert exr_diff_main([str(ref)]) == 2
