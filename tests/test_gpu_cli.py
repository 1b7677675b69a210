"""The reconstruction command line (bin/cudasirecon, the cudaSireconDriver loop:
SR_new_from_argv -> per time point setFile -> loadAndRescaleImage ->
setCurTimeIdx -> processOneVolume -> writeResult -> closeFiles) in TIFF mode:
an input folder, a file pattern, the OTF and a config file; results land in
<folder>/GPUsirecon/<name>_proc.tif (boostfs.cpp:59-72)."""
import os
import subprocess

import numpy as np
import pytest

import cudasirecon_gb300 as sr
from golden_cases import load, rel_l2

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EXE = os.path.join(ROOT, "cudasirecon_gb300", "bin", "cudasirecon")


def run_cli(args):
    r = subprocess.run([EXE] + args, capture_output=True, text=True, timeout=300)
    # like the reference's cudaSireconDriver, the program reports errors and still exits with 0
    assert r.returncode == 0 and "Error" not in r.stderr, r.stderr
    return r


def test_cli_tiff_folder_matches_reference(tmp_path):
    case, ref = load("c3d_64")
    data = tmp_path / "data"
    data.mkdir()
    sr.load_library()
    sr.write_tiff_float(str(data / "cell_t0.tif"), case["raw"][0].astype(np.float32))
    sr.write_tiff_float(str(data / "other.tif"), np.zeros((1, 4, 4), np.float32))  # does not match the pattern
    otf = tmp_path / "otf.tif"
    sr.write_tiff_float(str(otf), case["otf"])
    cfg = tmp_path / "config"
    cfg.write_text(case["config"])
    r = run_cli([str(data), "cell", str(otf), "-c", str(cfg)])
    assert "Time point 0, wave 0 done" in r.stdout
    out_dir = data / "GPUsirecon"
    assert sorted(os.listdir(out_dir)) == ["cell_t0_proc.tif"]
    got = sr.read_tiff_float(str(out_dir / "cell_t0_proc.tif"))
    want = ref["result"][0]
    assert got.shape == want.shape
    assert rel_l2(got, want) < 1e-4
    assert np.abs(got - want).max() / np.abs(want).max() < 1e-3


def test_cli_help_and_version():
    r = run_cli(["--help"])
    assert "cudasirecon" in r.stdout
    r = run_cli(["--version"])
    assert "Version" in r.stdout


def test_cli_reports_missing_otf(tmp_path):
    data = tmp_path / "data"
    data.mkdir()
    sr.load_library()
    sr.write_tiff_float(str(data / "cell_t0.tif"), np.zeros((15, 32, 32), np.float32))
    r = subprocess.run([EXE, str(data), "cell", str(tmp_path / "missing_otf.tif")], capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 0 and "Error" in r.stderr


def write_mrc(path, stack, dxy, dz, wave):
    """float32 [nz][ny][nx] as a DV/MRC file with the pixel sizes and the wavelength in the header"""
    import struct
    nz, ny, nx = stack.shape
    h = bytearray(1024)
    struct.pack_into("<4i", h, 0, nx, ny, nz, 2)
    struct.pack_into("<3f", h, 40, dxy, dxy, dz)
    struct.pack_into("<3i", h, 64, 1, 2, 3)
    struct.pack_into("<h", h, 96, -16224)
    struct.pack_into("<hh", h, 196, 1, wave)
    with open(path, "wb") as f:
        f.write(bytes(h))
        f.write(np.ascontiguousarray(stack, np.float32).tobytes())


def read_mrc(path):
    import struct
    with open(path, "rb") as f:
        h = f.read(1024)
        nx, ny, nz, mode = struct.unpack_from("<4i", h, 0)
        nxt = struct.unpack_from("<i", h, 92)[0]
        f.read(max(nxt, 0))
        assert mode == 2
        return np.frombuffer(f.read(4 * nx * ny * nz), np.float32).reshape(nz, ny, nx), h


def test_cli_mrc_input_and_output_match_reference(tmp_path):
    case, ref = load("c3d_64")
    inp, out = tmp_path / "cell.dv", tmp_path / "cell_proc.dv"
    write_mrc(inp, case["raw"][0].astype(np.float32), 0.08, 0.125, 528)
    otf = tmp_path / "otf.tif"
    sr.load_library()
    sr.write_tiff_float(str(otf), case["otf"])
    cfg = tmp_path / "config"
    cfg.write_text(case["config"])
    run_cli([str(inp), str(out), str(otf), "-c", str(cfg)])
    got, hdr = read_mrc(out)
    want = ref["result"][0]
    assert got.shape == want.shape
    assert rel_l2(got, want) < 1e-4
    assert np.abs(got - want).max() / np.abs(want).max() < 1e-3


def write_mrc_full(path, stack, dxy, dz, wave, labels, amean, ext_bytes=0):
    """DV/MRC input with labels, a mean and an extended header: fields the
    output header carries over or rewrites."""
    import struct
    nz, ny, nx = stack.shape
    h = bytearray(1024)
    struct.pack_into("<4i", h, 0, nx, ny, nz, 2)
    struct.pack_into("<3i", h, 28, nx, ny, nz)
    struct.pack_into("<3f", h, 40, dxy * nx, dxy * ny, dz * nz)
    struct.pack_into("<3f", h, 52, 90.0, 90.0, 90.0)
    struct.pack_into("<3i", h, 64, 1, 2, 3)
    struct.pack_into("<3f", h, 76, -3.5, 4321.0, amean)
    struct.pack_into("<i", h, 92, ext_bytes)
    struct.pack_into("<h", h, 96, -16224)
    struct.pack_into("<hh", h, 128, 0, 2)  # nint, nreal
    struct.pack_into("<hh", h, 180, 1, 0)  # num_times, interleaved
    struct.pack_into("<hh", h, 196, 1, wave)
    struct.pack_into("<3f", h, 208, 1.5, -2.25, 3.0)
    struct.pack_into("<i", h, 220, len(labels))
    for i, lab in enumerate(labels):
        h[224 + 80 * i:224 + 80 * i + len(lab)] = lab.encode()
    # xlen/ylen/zlen of a DV header are the pixel sizes (loadHeader reads dxy from ylen)
    struct.pack_into("<3f", h, 40, dxy, dxy, dz)
    with open(path, "wb") as f:
        f.write(bytes(h))
        f.write(bytes(range(256)) * (ext_bytes // 256) + bytes(ext_bytes % 256))
        f.write(np.ascontiguousarray(stack, np.float32).tobytes())


@pytest.mark.parametrize("title,nlab_in", [(False, 2), (True, 2), (False, 10), (True, 10)],
                         ids=["labels-kept", "long-title", "ten-labels", "long-title-ten-labels"])
def test_cli_mrc_output_header_every_field(tmp_path, title, nlab_in):
    """Every byte of the output header against the restatement of
    setOutputHeader, writeResult's min/max scan and saveCommandLineToHeader
    (oracle/mrc_header.py), with a title longer than 80 characters; label
    bytes the reference takes from uninitialised memory are skipped."""
    import struct
    from oracle.mrc_header import expected_header
    case, _ = load("c3d_64")
    labels = [f"input label {i} " + "x" * (20 + 3 * i) for i in range(nlab_in)]
    inp, out = tmp_path / "cell.dv", tmp_path / "cell_proc.dv"
    write_mrc_full(inp, case["raw"][0].astype(np.float32), 0.08, 0.125, 528, labels, amean=777.25, ext_bytes=512)
    otf = tmp_path / "otf.tif"
    sr.load_library()
    sr.write_tiff_float(str(otf), case["otf"])
    cfgdir = tmp_path / ("configuration_folder_with_a_long_name_" + "y" * 40)
    cfgdir.mkdir()
    cfg = cfgdir / "config"
    cfg.write_text(case["config"])
    extra = ["-c", str(cfg)] + (["--writeTitle"] if title else [])
    run_cli([str(inp), str(out), str(otf)] + extra)
    got, hdr = read_mrc(out)
    with open(inp, "rb") as f:
        in_hdr = f.read(1024)
    nz = got.shape[0]
    argv3 = [str(otf)] + extra  # the title starts at argv[3], the OTF file
    want, mask = expected_header(in_hdr, got, 2.0, 1, nz, argv3, title)
    if title:
        assert len(" ".join(argv3) + " ") > 80  # two title records
    assert hdr[:224] == want[:224], [i for i in range(224) if hdr[i] != want[i]]
    lab_got = np.frombuffer(hdr[224:], np.uint8)
    lab_want = np.frombuffer(want[224:], np.uint8)
    assert np.array_equal(lab_got[mask], lab_want[mask])
    nlab = struct.unpack_from("<i", hdr, 220)[0]
    assert nlab == (min(10, len(" ".join(argv3) + " ") // 80 + 1) + 1 if title else min(10, nlab_in + 1))


# --------------------------------------------------------------- debug dumps
# saveprefiltered / savealignedraw / saveoverlaps (cudaSirecon.cpp:270-287,
# 330-354, 433-445, 1179-1210, mrc.h:76-97): the intermediates are written,
# the volume is not reconstructed and no result is written.

def read_mrc_sections(path):
    """(data [nsec][ny][nx] float32 or complex64, header) of an MRC/DV file."""
    import struct
    with open(path, "rb") as f:
        h = f.read(1024)
        nx, ny, nz, mode = struct.unpack_from("<4i", h, 0)
        f.read(max(struct.unpack_from("<i", h, 92)[0], 0))
        body = f.read()
    dt = np.complex64 if mode == 4 else np.float32
    n = len(body) // (np.dtype(dt).itemsize * nx * ny)
    return np.frombuffer(body[:n * nx * ny * np.dtype(dt).itemsize], dt).reshape(n, ny, nx), h


def labels(h):
    import struct
    n = struct.unpack_from("<i", h, 220)[0]
    return [h[224 + 80 * i:304 + 80 * i].split(b"\0")[0].decode() for i in range(n)]


@pytest.fixture(scope="module")
def refmod():
    from oracle import build_ref
    if build_ref.build() is None:
        pytest.skip("the reference CUDA build could not be compiled")
    from oracle import refharness
    return refharness


def _mrc_case(tmp_path):
    case, _ = load("c3d_64")
    raw = case["raw"][0].astype(np.float32)
    inp = tmp_path / "cell.dv"
    write_mrc_full(inp, raw, 0.08, 0.125, 528, ["acquired"], amean=5.0)
    otf = tmp_path / "otf.tif"
    sr.load_library()
    sr.write_tiff_float(str(otf), case["otf"])
    cfg = tmp_path / "config"
    cfg.write_text(case["config"])
    return case, raw, inp, otf, cfg


def test_cli_saveprefiltered_writes_the_reference_bands_and_stops(tmp_path, refmod):
    import struct
    case, raw, inp, otf, cfg = _mrc_case(tmp_path)
    out, sep = tmp_path / "cell_proc.dv", tmp_path / "sep.dv"
    run_cli([str(inp), str(out), str(otf), "-c", str(cfg), "--saveprefiltered", str(sep)])
    assert os.path.getsize(out) == 1024  # header only: the volume was not reconstructed
    got, h = read_mrc_sections(sep)
    nx, ny = case["nx"], case["ny"]
    assert struct.unpack_from("<4i", h, 0) == (nx // 2 + 1, ny, raw.shape[0], 4)
    assert struct.unpack_from("<i", h, 92)[0] == 0
    assert struct.unpack_from("<3f", h, 76) == (0.0, 1.0, 0.0)
    assert labels(h) == ["acquired", "separated bands of all directions"]
    ref = refmod.RefRecon(nx, ny, raw.shape[0], case["config"], case["otf"])
    ref.set_raw(raw)
    ref.load_and_rescale(0)
    ref.set_cur_time(0)
    ref.stage_separate()
    nz = ref.nz
    assert got.shape[0] == 3 * 5 * nz
    for d in range(3):
        for b in range(5):
            want = ref.band(d, b)
            part = got[(d * 5 + b) * nz:(d * 5 + b + 1) * nz]
            assert rel_l2(part, want) < 2e-5, (d, b)
    ref.close()


def test_cli_saveoverlaps_writes_the_reference_overlaps_and_stops(tmp_path, refmod):
    import struct
    case, raw, inp, otf, cfg = _mrc_case(tmp_path)
    out, ovl = tmp_path / "cell_proc.dv", tmp_path / "ovl.dv"
    run_cli([str(inp), str(out), str(otf), "-c", str(cfg), "--saveoverlaps", str(ovl)])
    assert os.path.getsize(out) == 1024
    got, h = read_mrc_sections(ovl)
    nx, ny = case["nx"], case["ny"]
    ref = refmod.RefRecon(nx, ny, raw.shape[0], case["config"], case["otf"])
    ref.capture_overlaps(True)
    ref.set_raw(raw)
    ref.load_and_rescale(0)
    ref.set_cur_time(0)
    ref.stage_separate()
    ref.stage_fit()
    nz = ref.nz
    assert struct.unpack_from("<4i", h, 0) == (nx, ny, nz * 2 * 3, 4)
    assert struct.unpack_from("<hh", h, 180)[1] == 1 and struct.unpack_from("<h", h, 196)[0] == 2
    assert labels(h) == ["acquired", "overlaps in real space"]
    assert got.shape[0] == 3 * nz * 2  # per direction searched: z-interleaved overlap 0 / overlap 1 sections
    for d in range(3):
        o0, o1 = ref.captured_overlaps(d)
        part = got[d * 2 * nz:(d + 1) * 2 * nz]
        assert rel_l2(part[0::2], o0) < 1e-4, d
        assert rel_l2(part[1::2], o1) < 1e-4, d
    ref.close()


def test_cli_saveoverlaps_tiff_mode_keeps_the_last_direction(tmp_path, refmod):
    case, _ = load("c3d_64")
    raw = case["raw"][0].astype(np.float32)
    data = tmp_path / "data"
    data.mkdir()
    sr.load_library()
    sr.write_tiff_float(str(data / "cell_t0.tif"), raw)
    otf = tmp_path / "otf.tif"
    sr.write_tiff_float(str(otf), case["otf"])
    cfg = tmp_path / "config"
    cfg.write_text(case["config"])
    ovl = tmp_path / "ovl.tif"
    run_cli([str(data), "cell", str(otf), "-c", str(cfg), "--saveoverlaps", str(ovl)])
    assert not (data / "GPUsirecon" / "cell_t0_proc.tif").exists()
    got = sr.read_tiff_float(str(ovl))  # [2 nz][ny][2 nx] floats: overlap 0 planes, then overlap 1
    ref = refmod.RefRecon(case["nx"], case["ny"], raw.shape[0], case["config"], case["otf"])
    ref.capture_overlaps(True)
    ref.set_raw(raw)
    ref.load_and_rescale(0)
    ref.set_cur_time(0)
    ref.stage_separate()
    ref.stage_fit()
    o0, o1 = ref.captured_overlaps(2)
    c = got[..., 0::2] + 1j * got[..., 1::2]
    assert c.shape == (2 * ref.nz, case["ny"], case["nx"])
    assert rel_l2(c[:ref.nz], o0) < 1e-4 and rel_l2(c[ref.nz:], o1) < 1e-4
    ref.close()


def test_cli_savealignedraw_writes_a_header_and_stops(tmp_path):
    import struct
    case, raw, inp, otf, cfg = _mrc_case(tmp_path)
    out, al = tmp_path / "cell_proc.dv", tmp_path / "aligned.dv"
    run_cli([str(inp), str(out), str(otf), "-c", str(cfg), "--savealignedraw", str(al)])
    assert os.path.getsize(out) == 1024 and os.path.getsize(al) == 1024
    with open(al, "rb") as f:
        h = f.read()
    assert struct.unpack_from("<4i", h, 0) == (case["nx"], case["ny"], raw.shape[0], 2)
    assert labels(h) == ["acquired", "drift-corrected raw images"]
    assert struct.unpack_from("<3f", h, 76) == (-3.5, 4321.0, 5.0)  # the input header's min, max, mean
