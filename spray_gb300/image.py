"""HdrImage output: the PPM writer of SpRay's film mode
(src/display/image.h:183-204): P3, maximum 1023, rows written from the top
image row (y = H-1) down, each channel clamp(v * 1023, 0, 1023) truncated.
A NaN channel is written as 0, what the reference's unsigned conversion of
glm::clamp's NaN gives on its x86 build (the conversion itself is undefined)."""
from __future__ import annotations

import numpy as np


def ppm_bytes(rgba: np.ndarray) -> bytes:
    H, W = rgba.shape[:2]
    x = rgba[..., :3].astype(np.float32) * np.float32(1023.0)
    v = np.clip(np.where(np.isnan(x), np.float32(0.0), x), 0.0, 1023.0).astype(np.uint32)
    rows = v[::-1].reshape(-1, 3)
    body = "\n".join(f"{r} {g} {b}" for r, g, b in rows.tolist())
    return f"P3\n{W} {H}\n1023\n{body}\n".encode()


def write_ppm(path, rgba: np.ndarray) -> None:
    with open(path, "wb") as f:
        f.write(ppm_bytes(rgba))


def read_ppm_bytes(data: bytes) -> np.ndarray:
    """(H, W, 3) integer channels, row 0 = image row y = 0."""
    tok = data.split()
    assert tok[0] == b"P3"
    W, H = int(tok[1]), int(tok[2])
    return np.array(tok[4:], np.uint32).reshape(H, W, 3)[::-1]


def read_ppm(path) -> np.ndarray:
    with open(path, "rb") as f:
        return read_ppm_bytes(f.read())
