"""Regenerate the committed golden fixtures from the reference checkout.

Run once in a container that has the reference mounted (it reads the
reference's own checked-in goldens and mask PNGs); the GPU machine never runs it.

    python tests/golden/make_golden.py /root/reference

Writes into tests/golden/:

* ``tcc_golden.npz``      -- source/TCC_HLS/hls/tb/golden/tcc_expected_{r,i}.bin (81x81)
                             and the top-10 eigenvalues of kernels/kernel_info.txt
* ``image_golden.npz``    -- mask_256x256.bin (bit-packed, exactly 0/1) and
                             image_expected_512x512.bin (TCC-direct image, L=512)
* ``hls_golden.npz``      -- source/SOCS_HLS/data/hls_output_full_32.bin (32x32
                             tmpImgp, nk=4) and its mask, input/mask/
                             Different_resolution_tests/512x512.png / 255
* ``mask1024_t1.npz``     -- input/mask/1024x1024.png / 255, bit-packed (exactly 0/1)
"""
from __future__ import annotations

import os
import struct
import sys
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def read_png_gray8(path: str) -> np.ndarray:
    """Minimal decoder for 8-bit greyscale, non-interlaced PNG (the reference's mask format)."""
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n", path
    pos, idat = 8, b""
    w = h = None
    while pos < len(data):
        ln, typ = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + ln]
        pos += 12 + ln
        if typ == b"IHDR":
            w, h, bd, ct, _, _, il = struct.unpack(">IIBBBBB", body)
            assert bd == 8 and ct == 0 and il == 0, "only 8-bit grey, non-interlaced"
        elif typ == b"IDAT":
            idat += body
        elif typ == b"IEND":
            break
    raw = zlib.decompress(idat)
    out = np.zeros((h, w), dtype=np.uint8)
    prev = np.zeros(w, dtype=np.int32)
    stride = w + 1
    for y in range(h):
        f = raw[y * stride]
        line = np.frombuffer(raw, dtype=np.uint8, count=w, offset=y * stride + 1).astype(np.int32)
        cur = np.zeros(w, dtype=np.int32)
        if f == 0:
            cur = line
        elif f == 2:
            cur = (line + prev) & 255
        else:
            for x in range(w):
                a = cur[x - 1] if x > 0 else 0
                b = prev[x]
                c = prev[x - 1] if x > 0 else 0
                if f == 1:
                    p = a
                elif f == 3:
                    p = (a + b) >> 1
                else:  # Paeth
                    pa, pb, pc = abs(b - c), abs(a - c), abs(a + b - 2 * c)
                    p = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
                cur[x] = (line[x] + p) & 255
        out[y] = cur
        prev = cur
    return out


def main(ref: str) -> None:
    g = os.path.join(ref, "source/TCC_HLS/hls/tb/golden")
    tr = np.fromfile(os.path.join(g, "tcc_expected_r.bin"), np.float32).reshape(81, 81)
    ti = np.fromfile(os.path.join(g, "tcc_expected_i.bin"), np.float32).reshape(81, 81)
    eig = []
    for line in open(os.path.join(g, "kernels/kernel_info.txt")):
        if line.startswith("Eigenvalue"):
            eig.append(float(line.split(":")[1]))
    np.savez_compressed(os.path.join(HERE, "tcc_golden.npz"), tcc_r=tr, tcc_i=ti,
                        eigenvalues=np.asarray(eig, np.float64))

    m256 = np.fromfile(os.path.join(g, "mask_256x256.bin"), np.float32).reshape(256, 256)
    assert set(np.unique(m256)) <= {0.0, 1.0}
    img = np.fromfile(os.path.join(g, "image_expected_512x512.bin"), np.float32).reshape(512, 512)
    np.savez_compressed(os.path.join(HERE, "image_golden.npz"),
                        mask256_bits=np.packbits(m256.astype(np.uint8).ravel()), image512=img)

    d = os.path.join(ref, "source/SOCS_HLS/data")
    h32 = np.fromfile(os.path.join(d, "hls_output_full_32.bin"), np.float32).reshape(32, 32)
    h17 = np.fromfile(os.path.join(d, "hls_output_center_17.bin"), np.float32).reshape(17, 17)
    m512 = read_png_gray8(os.path.join(ref, "input/mask/Different_resolution_tests/512x512.png"))
    np.savez_compressed(os.path.join(HERE, "hls_golden.npz"), tmpimgp32=h32, center17=h17,
                        mask512_u8=m512)

    m1024 = read_png_gray8(os.path.join(ref, "input/mask/1024x1024.png"))
    assert set(np.unique(m1024)) <= {0, 255}
    np.savez_compressed(os.path.join(HERE, "mask1024_t1.npz"),
                        bits=np.packbits((m1024 // 255).astype(np.uint8).ravel()), shape=np.asarray(m1024.shape))
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("LITHO_REFERENCE_DIR", "/root/reference"))
