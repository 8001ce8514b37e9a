"""Writers for the glTF loader tests: PNG (every colour type and bit depth,
every filter type, optional Adam7), baseline JPEG (unit quantisers, the
example Huffman tables of the JPEG specification's Annex K), and small glTF
documents as .gltf + .bin, .gltf with data: URIs, and .glb."""
import base64
import json
import struct
import zlib

import numpy as np


# ----------------------------------------------------------------------------- PNG

def _chunk(tag, data):
    return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)


def _filter_rows(raw_rows, bpp):
    """Applies filter type (row index % 5) to each row of bytes."""
    out = []
    prev = bytes(len(raw_rows[0])) if raw_rows else b""
    for y, row in enumerate(raw_rows):
        ft = y % 5
        r = np.frombuffer(row, np.uint8).astype(np.int32)
        p = np.frombuffer(prev, np.uint8).astype(np.int32)
        a = np.concatenate([np.zeros(bpp, np.int32), r[:-bpp]]) if len(r) > bpp else np.zeros_like(r)
        c = np.concatenate([np.zeros(bpp, np.int32), p[:-bpp]]) if len(p) > bpp else np.zeros_like(p)
        if ft == 0:
            f = r
        elif ft == 1:
            f = r - a
        elif ft == 2:
            f = r - p
        elif ft == 3:
            f = r - (a + p) // 2
        else:
            pa, pb, pc = np.abs(p - c), np.abs(a - c), np.abs(a + p - 2 * c)
            pred = np.where((pa <= pb) & (pa <= pc), a, np.where(pb <= pc, p, c))
            f = r - pred
        out.append(bytes([ft]) + (f & 0xFF).astype(np.uint8).tobytes())
        prev = row
    return b"".join(out)


def _pack_samples(samples, depth):
    """Row of integer samples -> bytes (MSB-first for depth < 8, big-endian for 16)."""
    if depth == 8:
        return np.asarray(samples, np.uint8).tobytes()
    if depth == 16:
        return np.asarray(samples, ">u2").tobytes()
    bits = "".join(format(int(s), "0%db" % depth) for s in samples)
    bits += "0" * (-len(bits) % 8)
    return bytes(int(bits[i:i + 8], 2) for i in range(0, len(bits), 8))


def write_png(path, samples, ctype, depth, palette=None, trns=None, interlace=False):
    """samples: (h, w, channels) integer array in the file's sample values."""
    h, w, ch = samples.shape
    bpp = max(1, ch * depth // 8)
    passes = [(0, 0, 1, 1)] if not interlace else [(0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4),
                                                     (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2)]
    data = b""
    for (x0, y0, dx, dy) in passes:
        sub = samples[y0::dy, x0::dx]
        if sub.size == 0:
            continue
        rows = [_pack_samples(sub[y].reshape(-1), depth) for y in range(sub.shape[0])]
        data += _filter_rows(rows, bpp)
    png = b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, 1 if interlace else 0))
    if palette is not None:
        png += _chunk(b"PLTE", bytes(np.asarray(palette, np.uint8).reshape(-1)))
    if trns is not None:
        png += _chunk(b"tRNS", trns)
    png += _chunk(b"IDAT", zlib.compress(data, 6)) + _chunk(b"IEND", b"")
    with open(path, "wb") as f:
        f.write(png)


def pack_rgba(rgba):
    """(h, w, 4) uint8 -> R-in-MSB u32 texels."""
    r = rgba.astype(np.uint32)
    return ((r[..., 0] << 24) | (r[..., 1] << 16) | (r[..., 2] << 8) | r[..., 3]).reshape(-1)


# ---------------------------------------------------------------------------- JPEG

_ZZ = [0, 1, 8, 16, 9, 2, 3, 10, 17, 24, 32, 25, 18, 11, 4, 5, 12, 19, 26, 33, 40, 48, 41, 34, 27, 20, 13, 6, 7, 14,
       21, 28, 35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51, 58, 59, 52, 45, 38, 31, 39, 46, 53, 60,
       61, 54, 47, 55, 62, 63]
# Annex K.3 example tables (luminance DC / AC).
_DC_BITS = [0, 1, 5, 1, 1, 1, 1, 1, 1, 0, 0, 0, 0, 0, 0, 0]
_DC_VALS = list(range(12))
_AC_BITS = [0, 2, 1, 3, 3, 2, 4, 3, 5, 5, 4, 4, 0, 0, 1, 0x7D]
_AC_VALS = [
    0x01, 0x02, 0x03, 0x00, 0x04, 0x11, 0x05, 0x12, 0x21, 0x31, 0x41, 0x06, 0x13, 0x51, 0x61, 0x07, 0x22, 0x71, 0x14,
    0x32, 0x81, 0x91, 0xA1, 0x08, 0x23, 0x42, 0xB1, 0xC1, 0x15, 0x52, 0xD1, 0xF0, 0x24, 0x33, 0x62, 0x72, 0x82, 0x09,
    0x0A, 0x16, 0x17, 0x18, 0x19, 0x1A, 0x25, 0x26, 0x27, 0x28, 0x29, 0x2A, 0x34, 0x35, 0x36, 0x37, 0x38, 0x39, 0x3A,
    0x43, 0x44, 0x45, 0x46, 0x47, 0x48, 0x49, 0x4A, 0x53, 0x54, 0x55, 0x56, 0x57, 0x58, 0x59, 0x5A, 0x63, 0x64, 0x65,
    0x66, 0x67, 0x68, 0x69, 0x6A, 0x73, 0x74, 0x75, 0x76, 0x77, 0x78, 0x79, 0x7A, 0x83, 0x84, 0x85, 0x86, 0x87, 0x88,
    0x89, 0x8A, 0x92, 0x93, 0x94, 0x95, 0x96, 0x97, 0x98, 0x99, 0x9A, 0xA2, 0xA3, 0xA4, 0xA5, 0xA6, 0xA7, 0xA8, 0xA9,
    0xAA, 0xB2, 0xB3, 0xB4, 0xB5, 0xB6, 0xB7, 0xB8, 0xB9, 0xBA, 0xC2, 0xC3, 0xC4, 0xC5, 0xC6, 0xC7, 0xC8, 0xC9, 0xCA,
    0xD2, 0xD3, 0xD4, 0xD5, 0xD6, 0xD7, 0xD8, 0xD9, 0xDA, 0xE1, 0xE2, 0xE3, 0xE4, 0xE5, 0xE6, 0xE7, 0xE8, 0xE9, 0xEA,
    0xF1, 0xF2, 0xF3, 0xF4, 0xF5, 0xF6, 0xF7, 0xF8, 0xF9, 0xFA]


def _codes(bits, vals):
    code, k, out = 0, 0, {}
    for length in range(1, 17):
        for _ in range(bits[length - 1]):
            out[vals[k]] = (code, length)
            code += 1
            k += 1
        code <<= 1
    return out


class _BitWriter:
    def __init__(self):
        self.out = bytearray()
        self.acc = 0
        self.n = 0

    def put(self, v, n):
        for i in range(n - 1, -1, -1):
            self.acc = (self.acc << 1) | ((v >> i) & 1)
            self.n += 1
            if self.n == 8:
                self.out.append(self.acc)
                if self.acc == 0xFF:
                    self.out.append(0)
                self.acc = 0
                self.n = 0

    def flush(self):
        while self.n:
            self.put(1, 1)


def _cat(v):
    v = abs(v)
    return 0 if v == 0 else int(v).bit_length()


def _jpeg_blocks(rgb, subsample):
    """Component planes -> (sampling factors, per-component zigzag blocks
    [by][bx], MCU grid, padded block grid) with unit quantisers."""
    grey = rgb.ndim == 2
    h, w = rgb.shape[:2]
    x = rgb.astype(np.float64)
    if grey:
        planes = [x]
    else:
        r, g, b = x[..., 0], x[..., 1], x[..., 2]
        planes = [0.299 * r + 0.587 * g + 0.114 * b, -0.168736 * r - 0.331264 * g + 0.5 * b + 128,
                  0.5 * r - 0.418688 * g - 0.081312 * b + 128]
    hs = [2 if (subsample and i == 0) else 1 for i in range(len(planes))]
    hmax = max(hs)
    mw, mh = -(-w // (8 * hmax)), -(-h // (8 * hmax))
    C = np.array([[(np.sqrt(0.5) if u == 0 else 1.0) * np.cos((2 * xx + 1) * u * np.pi / 16) for xx in range(8)]
                  for u in range(8)]) / 2.0
    blocks = []
    for i, p in enumerate(planes):
        f = hs[i]
        pw, ph = mw * 8 * f, mh * 8 * f
        if f == 1 and hmax == 2:  # chroma at half resolution: average 2x2
            pad = np.pad(p, ((0, mh * 16 - h), (0, mw * 16 - w)), mode="edge")
            q = pad.reshape(mh * 8, 2, mw * 8, 2).mean(axis=(1, 3))
        else:
            q = np.pad(p, ((0, ph - h), (0, pw - w)), mode="edge")
        grid = []
        for by in range(mh * f):
            row = []
            for bx in range(mw * f):
                coef = np.rint(C @ (q[by * 8:by * 8 + 8, bx * 8:bx * 8 + 8] - 128.0) @ C.T).astype(int).reshape(-1)
                row.append([int(coef[_ZZ[k]]) for k in range(64)])
            grid.append(row)
        blocks.append(grid)
    return hs, hmax, blocks, mw, mh


def _seg(m, body):
    return bytes([0xFF, m]) + struct.pack(">H", len(body) + 2) + body


def write_jpeg(path, rgb, subsample=False, restart=0, progressive=False):
    """Baseline (or progressive) JPEG of (h, w, 3) uint8 (or (h, w) grey)
    with unit quantisers. Both forms carry the same coefficients, so a
    decoder must give them identical pixels."""
    h, w = rgb.shape[:2]
    hs, hmax, blocks, mw, mh = _jpeg_blocks(rgb, subsample)
    nc = len(blocks)
    out = b"\xff\xd8" + _seg(0xDB, bytes([0]) + bytes([1] * 64))
    sof = struct.pack(">BHHB", 8, h, w, nc)
    for i in range(nc):
        sof += bytes([i + 1, (hs[i] << 4) | hs[i], 0])
    out += _seg(0xC2 if progressive else 0xC0, sof)
    if progressive:
        out += _progressive_scans(h, w, hs, hmax, blocks, mw, mh, restart)
    else:
        out += _seg(0xC4, bytes([0x00]) + bytes(_DC_BITS) + bytes(_DC_VALS))
        out += _seg(0xC4, bytes([0x10]) + bytes(_AC_BITS) + bytes(_AC_VALS))
        if restart:
            out += _seg(0xDD, struct.pack(">H", restart))
        out += _baseline_scan(hs, blocks, mw, mh, restart)
    with open(path, "wb") as f:
        f.write(out + b"\xff\xd9")


def _baseline_scan(hs, blocks, mw, mh, restart):
    dc_codes, ac_codes = _codes(_DC_BITS, _DC_VALS), _codes(_AC_BITS, _AC_VALS)
    nc = len(blocks)
    bw = _BitWriter()
    pred = [0] * nc
    mcu = 0
    for my in range(mh):
        for mx in range(mw):
            if restart and mcu and mcu % restart == 0:
                bw.flush()
                bw.out += bytes([0xFF, 0xD0 + ((mcu // restart - 1) % 8)])
                pred = [0] * nc
            for ci in range(nc):
                f = hs[ci]
                for by in range(f):
                    for bx in range(f):
                        zz = blocks[ci][my * f + by][mx * f + bx]
                        d = zz[0] - pred[ci]
                        pred[ci] = zz[0]
                        s = _cat(d)
                        bw.put(*dc_codes[s])
                        if s:
                            bw.put(d if d > 0 else d + (1 << s) - 1, s)
                        run = 0
                        for k in range(1, 64):
                            v = zz[k]
                            if v == 0:
                                run += 1
                                continue
                            while run > 15:
                                bw.put(*ac_codes[0xF0])
                                run -= 16
                            s = _cat(v)
                            bw.put(*ac_codes[(run << 4) | s])
                            bw.put(v if v > 0 else v + (1 << s) - 1, s)
                            run = 0
                        if run:
                            bw.put(*ac_codes[0x00])
            mcu += 1
    bw.flush()
    sos = bytes([nc]) + b"".join(bytes([i + 1, 0x00]) for i in range(nc)) + bytes([0, 63, 0])
    return _seg(0xDA, sos) + bytes(bw.out)


# Progressive tables: every DC size 0-11 in 4 bits, every AC run/size symbol
# (runs 0-15, sizes 0-10: end-of-band runs, ZRL, coefficients) in 8 bits.
_PDC_BITS = [0, 0, 0, 12] + [0] * 12
_PDC_VALS = list(range(12))
_PAC_VALS = [(r << 4) | s for r in range(16) for s in range(11)]
_PAC_BITS = [0] * 7 + [len(_PAC_VALS)] + [0] * 8


def _progressive_scans(h, w, hs, hmax, blocks, mw, mh, restart):
    """Scans of T.81 Annex G: DC first (all components, Al 1), luma AC
    bands 1-5 and 6-63 at Al 2, chroma AC 1-63 at Al 1, luma AC refinement
    to Al 1, DC refinement, then every component's AC refinement to Al 0."""
    dc_codes, ac_codes = _codes(_PDC_BITS, _PDC_VALS), _codes(_PAC_BITS, _PAC_VALS)
    nc = len(blocks)
    out = _seg(0xC4, bytes([0x00]) + bytes(_PDC_BITS) + bytes(_PDC_VALS))
    out += _seg(0xC4, bytes([0x10]) + bytes(_PAC_BITS) + bytes(_PAC_VALS))
    if restart:
        out += _seg(0xDD, struct.pack(">H", restart))
    script = [(list(range(nc)), 0, 0, 0, 1)]
    if nc == 3:
        script += [([0], 1, 5, 0, 2), ([0], 6, 63, 0, 2), ([1], 1, 63, 0, 1), ([2], 1, 63, 0, 1),
                   ([0], 1, 63, 2, 1), (list(range(nc)), 0, 0, 1, 0), ([0], 1, 63, 1, 0), ([1], 1, 63, 1, 0),
                   ([2], 1, 63, 1, 0)]
    else:
        script += [([0], 1, 9, 0, 1), ([0], 10, 63, 0, 1), (list(range(nc)), 0, 0, 1, 0), ([0], 1, 63, 1, 0)]
    for comps, ss, se, ah, al in script:
        out += _progressive_scan(h, w, hs, hmax, blocks, mw, mh, restart, comps, ss, se, ah, al, dc_codes, ac_codes)
    return out


def _progressive_scan(h, w, hs, hmax, blocks, mw, mh, restart, comps, ss, se, ah, al, dc_codes, ac_codes):
    bw = _BitWriter()
    st = {"eobrun": 0, "be": []}
    pred = {c: 0 for c in comps}

    def emit_eobrun():
        n = st["eobrun"]
        if n > 0:
            nb = n.bit_length() - 1
            bw.put(*ac_codes[nb << 4])
            if nb:
                bw.put(n & ((1 << nb) - 1), nb)
            for bit in st["be"]:
                bw.put(bit, 1)
            st["eobrun"], st["be"] = 0, []

    def block(ci, zz):
        if ss == 0:
            if ah == 0:
                v = zz[0] >> al
                d = v - pred[ci]
                pred[ci] = v
                s = _cat(d)
                bw.put(*dc_codes[s])
                if s:
                    bw.put(d if d > 0 else d + (1 << s) - 1, s)
            else:
                bw.put((zz[0] >> al) & 1, 1)
            return
        if ah == 0:
            r = 0
            for k in range(ss, se + 1):
                a = abs(zz[k]) >> al
                if a == 0:
                    r += 1
                    continue
                emit_eobrun()
                while r > 15:
                    bw.put(*ac_codes[0xF0])
                    r -= 16
                s = a.bit_length()
                bw.put(*ac_codes[(r << 4) | s])
                bw.put(a if zz[k] > 0 else (~a) & ((1 << s) - 1), s)
                r = 0
            if r > 0:
                st["eobrun"] += 1
                if st["eobrun"] == 0x7FFF:
                    emit_eobrun()
            return
        absv = [abs(zz[k]) >> al for k in range(64)]
        eob = 0
        for k in range(ss, se + 1):
            if absv[k] == 1:
                eob = k
        r, br = 0, []
        for k in range(ss, se + 1):
            a = absv[k]
            if a == 0:
                r += 1
                continue
            while r > 15 and k <= eob:
                emit_eobrun()
                bw.put(*ac_codes[0xF0])
                r -= 16
                for bit in br:
                    bw.put(bit, 1)
                br = []
            if a > 1:
                br.append(a & 1)
                continue
            emit_eobrun()
            bw.put(*ac_codes[(r << 4) | 1])
            bw.put(1 if zz[k] > 0 else 0, 1)
            for bit in br:
                bw.put(bit, 1)
            br, r = [], 0
        if r > 0 or br:
            st["eobrun"] += 1
            st["be"] += br
            if st["eobrun"] == 0x7FFF or len(st["be"]) > 900:
                emit_eobrun()

    units = []
    if len(comps) == 1:
        c = comps[0]
        cw, chh = -(-w * hs[c] // hmax), -(-h * hs[c] // hmax)
        for by in range(-(-chh // 8)):
            for bx in range(-(-cw // 8)):
                units.append([(c, by, bx)])
    else:
        for my in range(mh):
            for mx in range(mw):
                units.append([(c, my * hs[c] + by, mx * hs[c] + bx) for c in comps
                              for by in range(hs[c]) for bx in range(hs[c])])
    for u, unit in enumerate(units):
        if restart and u and u % restart == 0:
            emit_eobrun()
            bw.flush()
            bw.out += bytes([0xFF, 0xD0 + ((u // restart - 1) % 8)])
            pred = {c: 0 for c in comps}
        for c, by, bx in unit:
            block(c, blocks[c][by][bx])
    emit_eobrun()
    bw.flush()
    sos = bytes([len(comps)]) + b"".join(bytes([c + 1, 0x00]) for c in comps) + bytes([ss, se, (ah << 4) | al])
    return _seg(0xDA, sos) + bytes(bw.out)


# ---------------------------------------------------------------------------- glTF

class DocBuilder:
    """Accumulates one binary buffer and the JSON of a glTF document."""

    def __init__(self):
        self.bin = bytearray()
        self.doc = {"asset": {"version": "2.0"}, "scenes": [{"nodes": []}], "scene": 0, "nodes": [], "meshes": [],
                    "accessors": [], "bufferViews": [], "buffers": []}

    def accessor(self, arr, comp, type_, normalized=False, stride=0):
        a = np.ascontiguousarray(arr)
        while len(self.bin) % 4:
            self.bin.append(0)
        off = len(self.bin)
        data = a.tobytes()
        if stride:
            elem = a.dtype.itemsize * (a.shape[1] if a.ndim > 1 else 1)
            rows = [data[i * elem:(i + 1) * elem] + bytes(stride - elem) for i in range(a.shape[0])]
            data = b"".join(rows)
        self.bin += data
        view = {"buffer": 0, "byteOffset": off, "byteLength": len(data)}
        if stride:
            view["byteStride"] = stride
        self.doc["bufferViews"].append(view)
        acc = {"bufferView": len(self.doc["bufferViews"]) - 1, "componentType": comp,
               "count": int(a.shape[0]), "type": type_}
        if normalized:
            acc["normalized"] = True
        self.doc["accessors"].append(acc)
        return len(self.doc["accessors"]) - 1

    def write(self, base, form):
        """form: 'bin' (.gltf + .bin), 'data' (.gltf with a data: URI), 'glb'."""
        doc = json.loads(json.dumps(self.doc))
        binary = bytes(self.bin)
        if form == "bin":
            doc["buffers"] = [{"uri": "geom data.bin".replace(" ", "%20"), "byteLength": len(binary)}]
            with open(base + ".gltf", "w") as f:
                json.dump(doc, f)
            with open(base.rsplit("/", 1)[0] + "/geom data.bin", "wb") as f:
                f.write(binary)
            return base + ".gltf"
        if form == "data":
            doc["buffers"] = [{"uri": "data:application/octet-stream;base64," + base64.b64encode(binary).decode(),
                               "byteLength": len(binary)}]
            with open(base + ".gltf", "w") as f:
                json.dump(doc, f)
            return base + ".gltf"
        doc["buffers"] = [{"byteLength": len(binary)}]
        js = json.dumps(doc).encode()
        js += b" " * (-len(js) % 4)
        bn = binary + bytes(-len(binary) % 4)
        body = struct.pack("<II", len(js), 0x4E4F534A) + js + struct.pack("<II", len(bn), 0x004E4942) + bn
        with open(base + ".glb", "wb") as f:
            f.write(struct.pack("<III", 0x46546C67, 2, 12 + len(body)) + body)
        return base + ".glb"
