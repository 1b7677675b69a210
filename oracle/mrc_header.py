"""Test infrastructure (oracle): the reference's output MRC/DV header,
restated from its source, for checking the product's CLI output byte for
byte.

Follows
  * setOutputHeader, src/cudaSirecon/mrc.h:47-60 (mode float, sizes scaled by
    the zoom factors, pixel sizes divided by them, inbsym = 0);
  * SIM_Reconstructor::writeResult, src/cudaSirecon/cudaSirecon.cpp:1663-1689
    (amin/amax of time point 0 with the `else if` update: the minimum only
    moves on values that do not raise the maximum);
  * saveCommandLineToHeader, src/cudaSirecon/mrc.h:62-74, whose two Priism
    IM-library calls are restated from that library's documented behaviour
    (the library is not in the reference tree): IMAlLab(titles,
    strlen(titles)/80 + 1) replaces the labels with 80-byte records of the
    title string (the arguments after the three positional ones, each
    followed by a space); IMWrHdr(header.label, ntflag = 1, amin, amax,
    amean) appends the kept header's first label -- the input file's -- and
    drops the oldest label when all ten are in use.

The reference copies the title records from a 1000-byte stack buffer, so the
bytes after the string's terminator are uninitialised there; this oracle
writes zeros and `label_mask` marks them so a comparison can skip them.
"""
import struct

import numpy as np

FLT_MAX = float(np.finfo(np.float32).max)


def minmax_else_if(vol: np.ndarray):
    """writeResult's scan (cudaSirecon.cpp:1676-1680): max updated first, min
    only in the `else` branch, both starting from -/+FLT_MAX, in section
    order."""
    v = np.ascontiguousarray(vol, np.float32).ravel()
    maxv, minv = np.float32(-FLT_MAX), np.float32(FLT_MAX)
    # vectorised form of the sequential loop: a value updates the maximum iff
    # it exceeds every value before it (and -FLT_MAX); it updates the minimum
    # iff it does not update the maximum and is below every earlier minimum
    # candidate
    run_max = np.maximum.accumulate(np.concatenate([[maxv], v]))[:-1]
    raises_max = v > run_max
    # NaNs compare false both ways: they move neither value
    cand = np.where(raises_max | np.isnan(v), np.float32(FLT_MAX), v)
    if cand.size:
        minv = min(minv, np.float32(cand.min()))
    if v.size and not np.isnan(v).all():
        maxv = max(maxv, np.float32(np.nanmax(v)))
    return float(minv), float(maxv)


def expected_header(in_hdr: bytes, out_vol: np.ndarray, zoom: float, z_zoom: int, nz_per_volume: int,
                    argv_from_3: list, write_title: bool):
    """(header bytes, label_mask) of the output file.  in_hdr: the input's
    1024 header bytes (little endian); out_vol: time point 0's result;
    argv_from_3: the command line from argv[3] on (the OTF file, then the
    options), which saveCommandLineToHeader joins into the title."""
    h = bytearray(in_hdr[:1024])
    nx, ny = struct.unpack_from("<2i", h, 0)
    xlen, ylen, zlen = struct.unpack_from("<3f", h, 40)
    nwaves = max(1, struct.unpack_from("<h", h, 196)[0])
    ntimes = max(1, struct.unpack_from("<h", h, 180)[0])
    f32 = np.float32
    struct.pack_into("<i", h, 12, 2)  # IW_FLOAT
    struct.pack_into("<i", h, 8, nz_per_volume * nwaves * ntimes * z_zoom)
    struct.pack_into("<i", h, 0, int(f32(nx) * f32(zoom)))
    struct.pack_into("<i", h, 4, int(f32(ny) * f32(zoom)))
    struct.pack_into("<3f", h, 40, f32(xlen) / f32(zoom), f32(ylen) / f32(zoom), f32(zlen) / f32(z_zoom))
    struct.pack_into("<i", h, 92, 0)  # inbsym: no extended header
    amin, amax = minmax_else_if(out_vol)
    struct.pack_into("<2f", h, 76, amin, amax)
    mask = np.ones(800, bool)  # which label bytes are determined
    first_in_label = bytes(in_hdr[224:304])
    nlab = struct.unpack_from("<i", h, 220)[0]
    if write_title:
        titles = "".join(a + " " for a in argv_from_3).encode()[:999]
        nl = min(10, len(titles) // 80 + 1)
        buf = titles + b"\0" * (1000 - len(titles))
        h[224:1024] = b"\0" * 800
        for i in range(nl):
            h[224 + 80 * i:304 + 80 * i] = buf[80 * i:80 * (i + 1)]
        mask[:] = True
        mask[len(titles) + 1:80 * nl] = False  # uninitialised in the reference
        nlab = nl
    nlab = max(nlab, 0)
    if nlab >= 10:
        h[224:944] = h[304:1024]
        mask[:720] = mask[80:800].copy()
        nlab = 9
    h[224 + 80 * nlab:304 + 80 * nlab] = first_in_label
    mask[80 * nlab:80 * nlab + 80] = True
    if write_title:  # whether IMAlLab clears the records it does not write is not known
        mask[80 * (nlab + 1):] = False
    struct.pack_into("<i", h, 220, nlab + 1)
    return bytes(h), mask
