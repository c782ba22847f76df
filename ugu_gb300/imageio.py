"""Host writers for the images a render produces.

WriteFaceIdAsText (src/util/io_util.cc:22-33): one face id per line, rows
top to bottom.  ugu writes its 8-bit images as PNG through stb
(src/image_io.cc), which is not available here; these write the binary
netpbm formats instead (P5 gray, P6 RGB; 16-bit big-endian for 16-bit
depth, as the format requires) and PFM for float images, which any image
viewer or numpy reads back."""
from __future__ import annotations

import numpy as np


def WriteFaceIdAsText(face_id: np.ndarray, path: str) -> None:
    ids = np.ascontiguousarray(face_id, np.int32).reshape(-1)
    with open(path, "w") as f:
        if ids.size:
            f.write("\n".join(map(str, ids.tolist())))
            f.write("\n")


def write_pnm(path: str, img: np.ndarray) -> None:
    """uint8 or uint16, H x W (P5) or H x W x 3 (P6)."""
    img = np.asarray(img)
    if img.dtype not in (np.uint8, np.uint16) or img.ndim not in (2, 3):
        raise ValueError("write_pnm: uint8/uint16 H x W or H x W x 3 expected")
    if img.ndim == 3 and img.shape[2] != 3:
        raise ValueError("write_pnm: 3 channels expected")
    H, W = img.shape[:2]
    magic = b"P6" if img.ndim == 3 else b"P5"
    maxval = 255 if img.dtype == np.uint8 else 65535
    data = np.ascontiguousarray(img.astype(">u2") if img.dtype == np.uint16 else img)
    with open(path, "wb") as f:
        f.write(magic + b"\n%d %d\n%d\n" % (W, H, maxval))
        f.write(data.tobytes())


def write_pfm(path: str, img: np.ndarray) -> None:
    """float32, H x W ('Pf') or H x W x 3 ('PF'); little-endian, rows
    stored bottom to top as the format defines."""
    img = np.asarray(img, np.float32)
    if img.ndim == 3 and img.shape[2] != 3:
        raise ValueError("write_pfm: 1 or 3 channels expected")
    H, W = img.shape[:2]
    magic = b"PF" if img.ndim == 3 else b"Pf"
    with open(path, "wb") as f:
        f.write(magic + b"\n%d %d\n-1.0\n" % (W, H))
        f.write(np.ascontiguousarray(img[::-1]).astype("<f4").tobytes())


def _header(data: bytes):
    """The three header lines these writers emit, and the binary body."""
    magic, size, third, body = data.split(b"\n", 3)
    W, H = (int(x) for x in size.split())
    return magic, W, H, third, body


def read_pnm(path: str) -> np.ndarray:
    with open(path, "rb") as f:
        magic, W, H, maxval, body = _header(f.read())
    maxval = int(maxval)
    dt = np.uint8 if maxval < 256 else np.dtype(">u2")
    shape = (H, W, 3) if magic == b"P6" else (H, W)
    return np.frombuffer(body, dt).reshape(shape).astype(np.uint8 if maxval < 256 else np.uint16)


def read_pfm(path: str) -> np.ndarray:
    with open(path, "rb") as f:
        magic, W, H, scale, body = _header(f.read())
    dt = "<f4" if float(scale) < 0 else ">f4"
    shape = (H, W, 3) if magic == b"PF" else (H, W)
    return np.frombuffer(body, dt).reshape(shape)[::-1].astype(np.float32)
