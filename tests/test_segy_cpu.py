"""The SEG-Y writer (host code of the post-stack chain) without a GPU: headers
and samples read back by an independent reader of the SEG-Y rev 1 layout."""
import struct

import numpy as np

from rtm_gpu_gb300 import capi


def ibm(f):
    """IEEE single -> IBM single bits (independent reference: hex digits of
    the magnitude, truncated)."""
    f = float(np.float32(f))
    if f == 0.0:
        return struct.unpack(">I", struct.pack(">f", f))[0] & 0x80000000
    s = 0x80000000 if f < 0 else 0
    m, e = abs(f), 0
    while m >= 1.0:
        m /= 16.0
        e += 1
    while m < 1.0 / 16.0:
        m *= 16.0
        e -= 1
    frac = int(m * (1 << 24))  # truncation
    return s | ((e + 64) << 24) | frac


def write(path, data, template=None, dt=10.0):
    ntr, ns = data.shape
    sx = np.arange(ntr, dtype=np.float32) * 10
    sy = -sx
    off = (1000 - np.arange(ntr)).astype(np.float32)
    rc = capi.lib().rtm_write_segy(str(path).encode(), None if template is None else str(template).encode(),
                                   capi.fptr(np.ascontiguousarray(data)), ntr, ns, dt, capi.fptr(sx),
                                   capi.fptr(sy), 1.0, 1.0, capi.fptr(off))
    assert rc == 0
    return open(path, "rb").read()


def test_ieee_without_template(product_lib, tmp_path):
    data = np.random.default_rng(1).standard_normal((5, 37)).astype(np.float32)
    b = write(tmp_path / "a.sgy", data)
    assert len(b) == 3600 + 5 * (240 + 37 * 4)
    dt, ns, fmt = struct.unpack(">h", b[3216:3218])[0], struct.unpack(">h", b[3220:3222])[0], \
        struct.unpack(">h", b[3224:3226])[0]
    assert (dt, ns, fmt) == (10000, 37, 5)
    for i in range(5):
        h = b[3600 + i * (240 + 148):]
        off, sx, sy, gx, gy = struct.unpack(">i", h[36:40])[0], *struct.unpack(">iiii", h[72:88])
        assert (off, sx, sy, gx, gy) == (1000 - i, 10 * i, -10 * i, 1, 1)
        vals = np.frombuffer(h[240:240 + 148], ">f4")
        assert np.array_equal(vals, data[i])


def test_ibm_template_headers_kept(product_lib, tmp_path):
    tpl = bytearray(3600 + 240)
    tpl[0:3200] = bytes([0xC1]) * 3200  # EBCDIC 'A'
    tpl[3200 + 24:3200 + 26] = struct.pack(">h", 1)  # IBM floats
    tpl[3200 + 100:3200 + 102] = struct.pack(">h", 77)  # a field the writer keeps
    tpl[3600 + 0:3600 + 4] = struct.pack(">i", 42)  # tracl of the template trace
    (tmp_path / "SGY_Model.sgy").write_bytes(bytes(tpl))
    data = np.array([[0.0, 1.0, -1.5, 3.14159, 1e-30, -2.5e20, 0.1, 65504.0]], np.float32)
    b = write(tmp_path / "b.sgy", data, tmp_path / "SGY_Model.sgy", dt=12.0)
    assert b[:3200] == bytes([0xC1]) * 3200
    assert struct.unpack(">h", b[3300:3302])[0] == 77
    assert struct.unpack(">h", b[3216:3218])[0] == 12000
    assert struct.unpack(">i", b[3600:3604])[0] == 42
    words = struct.unpack(">8I", b[3840:3840 + 32])
    assert list(words) == [ibm(x) for x in data[0]]
