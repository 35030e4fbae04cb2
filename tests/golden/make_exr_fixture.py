"""Writes tests/golden/exr_2x2.bin: the bytes of a 2 x 2 RGB float image as an OpenEXR file,
spelled out field by field from the OpenEXR file-layout specification ("OpenEXR File Layout"):

  magic number 20000630 (bytes 76 2f 31 01), version field 2 (single-part scanline, short names);
  header: attributes "name\\0 type\\0 size(int32) value", alphabetical here, ended by a 0 byte:
    channels (chlist: per channel "name\\0 pixel_type(int32: 2 = FLOAT) pLinear(uchar) 3 reserved
      bytes xSampling(int32) ySampling(int32)", ended by a 0 byte; channels in name order B, G, R),
    compression (uchar 0 = NO_COMPRESSION), dataWindow and displayWindow (box2i: xMin yMin xMax
    yMax), lineOrder (uchar 0 = INCREASING_Y), pixelAspectRatio (float 1), screenWindowCenter
    (v2f 0 0), screenWindowWidth (float 1);
  line offset table: one uint64 per scanline block (one scanline per block, uncompressed),
    each the file offset of its block;
  scanline blocks: y (int32), data size (int32), then for each channel in name order the
    scanline's samples (float32, little endian).

It does not call the library's writer.  Run:  python tests/golden/make_exr_fixture.py
"""
import struct
from pathlib import Path

HERE = Path(__file__).resolve().parent

W, H = 2, 2
# pixel (x, y): R = 1 + x + 2y, G = 10 R, B = 100 R
R = [[1.0 + x + 2 * y for x in range(W)] for y in range(H)]


def attr(name: str, typ: str, value: bytes) -> bytes:
    return name.encode() + b"\0" + typ.encode() + b"\0" + struct.pack("<i", len(value)) + value


def main():
    chlist = b"".join(c.encode() + b"\0" + struct.pack("<i", 2) + bytes([0, 0, 0, 0]) + struct.pack("<ii", 1, 1)
                      for c in ("B", "G", "R")) + b"\0"
    box = struct.pack("<iiii", 0, 0, W - 1, H - 1)
    header = (struct.pack("<I", 20000630) + struct.pack("<I", 2) +
              attr("channels", "chlist", chlist) +
              attr("compression", "compression", bytes([0])) +
              attr("dataWindow", "box2i", box) +
              attr("displayWindow", "box2i", box) +
              attr("lineOrder", "lineOrder", bytes([0])) +
              attr("pixelAspectRatio", "float", struct.pack("<f", 1.0)) +
              attr("screenWindowCenter", "v2f", struct.pack("<ff", 0.0, 0.0)) +
              attr("screenWindowWidth", "float", struct.pack("<f", 1.0)) +
              b"\0")
    blocks = []
    for y in range(H):
        data = b"".join(struct.pack("<f", s * R[y][x]) for s in (100.0, 10.0, 1.0) for x in range(W))
        blocks.append(struct.pack("<ii", y, len(data)) + data)
    table_end = len(header) + 8 * H
    offsets, off = [], table_end
    for b in blocks:
        offsets.append(struct.pack("<Q", off))
        off += len(b)
    (HERE / "exr_2x2.bin").write_bytes(header + b"".join(offsets) + b"".join(blocks))


if __name__ == "__main__":
    main()
