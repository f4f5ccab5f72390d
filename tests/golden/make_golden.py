"""Generates the golden vectors under tests/golden from the reference's own
sources.  Run in a tree where the reference is mounted (it builds
oracle/_ref/refshim_harness from the reference's src/threshold.cpp,
src/segmentation.cpp, src/find_boundaries.cpp, src/fit_quad.cpp and
include/*.h; see oracle/refshim/).

Writes:
  reference_images.npz  the reference's three input PNGs, decoded
  small_frames.npz      small hand-made and synthetic frames
  records.npz           record helpers (Combinadics decode, calc_theta,
                        ClusterBounds::cx/cy/dot, ValidBlobFilter,
                        compute_initial_linefit, fit_line, get_moment) on
                        seeded inputs
  pipeline.json         per frame and per stage: element count and SHA-256 of
                        the canonical bytes (record padding excluded)
  colour.npz            colour removal as the reference's loader does it: seeded
                        grey + alpha, RGB and RGBA images encoded with the
                        reference's vendored stb_image_write.h and decoded with
                        its stb_image.h to one channel (oracle/_ref/stb_grey)
"""
import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "sycl-apriltag-test_gb300"))

import golden_io  # noqa: E402

# the reference tree: ATAG_REFERENCE_TREE, else a checkout named "reference"
# beside this repository
REF = os.environ.get("ATAG_REFERENCE_TREE") or os.path.normpath(
    os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "..", "..", "reference"))


def small_frames():
    from atag import synth
    rng = np.random.default_rng(7)
    out = {
        "noise_64": rng.integers(0, 256, (64, 64), dtype=np.uint8),
        "noise_68x132": rng.integers(0, 256, (68, 132), dtype=np.uint8),
        "checker_96x128": ((np.indices((96, 128)).sum(0) // 8) % 2 * 255).astype(np.uint8),
        "flat_32": np.full((32, 32), 100, np.uint8),
        "tiny_4x4": rng.integers(0, 256, (4, 4), dtype=np.uint8),
    }
    b = rng.integers(0, 2, (20, 28)).astype(np.uint8) * 255
    out["blocky_80x112"] = np.kron(b, np.ones((4, 4), np.uint8))
    sq = np.full((120, 160), 230, np.uint8)
    sq[30:90, 50:110] = 20
    sq[45:75, 65:95] = 230
    out["square_120x160"] = sq
    for seed in (1, 2, 3):
        img = synth.render(synth.CONFIGS["vga"], seed)
        out[f"vga_seed{seed}_d2"] = np.ascontiguousarray(img[::2, ::2])
    return out


def colour_cases():
    """Seeded 2/3/4-channel images: uniform noise, and a synthetic frame
    tinted per channel (so the luma weights matter)."""
    from atag import synth
    rng = np.random.default_rng(11)
    out = {}
    for c in (2, 3, 4):
        out[f"noise_c{c}"] = rng.integers(0, 256, (48, 64, c), dtype=np.uint8)
    grey = synth.render(synth.CONFIGS["vga"], 4)[100:220, 200:360].astype(np.int32)
    for c in (3, 4):
        chans = [np.clip(grey * rng.uniform(0.6, 1.2) + rng.integers(-40, 40), 0, 255) for _ in range(c)]
        out[f"tinted_c{c}"] = np.stack(chans, axis=-1).astype(np.uint8)
    return out


def run_stb_grey(tool, img, tmp):
    h, w, c = img.shape
    np.ascontiguousarray(img).tofile(os.path.join(tmp, "c.raw"))
    subprocess.run([tool, os.path.join(tmp, "c.raw"), str(w), str(h), str(c), os.path.join(tmp, "g.raw")],
                   check=True, capture_output=True)
    return np.fromfile(os.path.join(tmp, "g.raw"), dtype=np.uint8).reshape(h, w)


def run_pipeline(harness, img, tmp):
    img.tofile(os.path.join(tmp, "in.raw"))
    subprocess.run([harness, os.path.join(tmp, "in.raw"), str(img.shape[1]), str(img.shape[0]), tmp], check=True,
                   capture_output=True)
    out = {}
    for name, dtype in golden_io.PIPELINE_ARRAYS.items():
        a = np.fromfile(os.path.join(tmp, name + ".bin"), dtype=dtype)
        out[name] = {"n": int(len(a)), "sha256": golden_io.digest(a)}
    return out


def main():
    sys.path.insert(0, os.path.join(ROOT, "oracle", "refshim"))
    import build_refshim
    harness = build_refshim.build()
    if harness is None:
        raise SystemExit(f"reference tree not found at {REF}")
    from pngdecode import read_png_grey
    imgs = {n[:-4]: read_png_grey(os.path.join(REF, n)) for n in ("decimate.png", "decimate4.png", "decimate2.png")}
    np.savez_compressed(os.path.join(HERE, "reference_images.npz"), **imgs)
    small = small_frames()
    np.savez_compressed(os.path.join(HERE, "small_frames.npz"), **small)
    pipeline = {}
    with tempfile.TemporaryDirectory() as tmp:
        for name, img in list(imgs.items()) + list(small.items()):
            pipeline[name] = run_pipeline(harness, img, tmp)
        subprocess.run([harness, "--records", tmp], check=True, capture_output=True)
        rec = {name: np.fromfile(os.path.join(tmp, name + ".bin"), dtype=dt)
               for name, dt in golden_io.RECORD_ARRAYS.items()}
    np.savez_compressed(os.path.join(HERE, "records.npz"), **rec)
    stb = build_refshim.build_stb_grey()
    colour = {}
    with tempfile.TemporaryDirectory() as tmp:
        for name, img in colour_cases().items():
            colour[name] = img
            colour[name + "_grey"] = run_stb_grey(stb, img, tmp)
    np.savez_compressed(os.path.join(HERE, "colour.npz"), **colour)
    with open(os.path.join(HERE, "pipeline.json"), "w") as f:
        json.dump(pipeline, f, indent=1, sort_keys=True)
    print("golden vectors written:", ", ".join(sorted(pipeline)))


if __name__ == "__main__":
    main()
