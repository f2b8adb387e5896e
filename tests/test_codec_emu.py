"""The LZ4 and zstd encoder kernels, run on the CPU under the SIMT emulation
of tests/emu (AddressSanitizer + UBSan alignment checks when the compiler
has them), with every chunk decoded by the stock liblz4 / libzstd."""
import os
import shutil
import subprocess

import pytest

import harness as H

EMU = os.path.join(H.ROOT, "tests", "emu")
BIN = os.path.join(EMU, "_build", "codec_emu")


@pytest.fixture(scope="module")
def emu():
    if not shutil.which("g++"):
        pytest.skip("g++ not available")
    if not (H.oracle().oracle_codecs_available() & 3) == 3:
        pytest.skip("stock liblz4/libzstd not available")
    os.makedirs(os.path.dirname(BIN), exist_ok=True)
    base = ["g++", "-std=c++20", "-O1", "-g", "-I", os.path.join(EMU, "fake"),
            "-I", os.path.join(H.ROOT, "include"),
            "-I", os.path.join(H.ROOT, "chucky_gb300", "csrc"),
            os.path.join(EMU, "codec_emu.cpp"), os.path.join(EMU, "simt.cpp"),
            "-o", BIN, "-ldl", "-lpthread"]
    san = ["-fsanitize=address,undefined", "-fno-sanitize-recover=all"]
    r = subprocess.run(base[:1] + san + base[1:], capture_output=True, text=True)
    if r.returncode != 0:  # no sanitizer runtime: plain build
        r = subprocess.run(base, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return BIN


CASES = [(1024, 6), (37, 3), (13, 2), (1, 2)]
BIG = [("zstd", "xor16", 200000, 1), ("zstd", "mixed", 131072, 2),
       ("lz4", "xor16", 140000, 1), ("lz4", "mixed", 65536, 2),
       # skewed bytes: Huffman depths beyond the 11-bit limit get repaired
       ("zstd", "geom", 40000, 1), ("lz4", "geom", 9000, 1),
       # FSE-coded Huffman weights (more than 128), both parities of their
       # count (the two interleaved state chains end on either state)
       ("zstd", "u200", 70000, 1), ("zstd", "u201", 70000, 1),
       # more than 32 segments per chunk, whole groups of 32 segments
       # without a match before and after ones with matches
       ("lz4", "halves", 300000, 2), ("lz4", "random", 270000, 1)]


# The higher levels: the wide match window (region tables of earlier regions
# probed by the parse) and, for zstd, FSE-described sequence tables in the
# chunk's first block with sequences, repeated by every later block.
WIDE = [("lz4", "xor16", 40000, 1, 2), ("lz4", "mixed", 65536, 2, 2),
        ("lz4", "halves", 70000, 2, 2), ("lz4", "geom", 9000, 1, 2),
        ("zstd", "xor16", 40000, 1, 3), ("zstd", "mixed", 131072, 2, 3),
        ("zstd", "geom", 20000, 1, 3), ("zstd", "u200", 70000, 1, 3),
        ("zstd", "halves", 70000, 2, 3)]
WIDE_SMALL = [(1024, 6), (37, 3), (1, 2)]
REFS = [("zstd", "mixed", 70000, 3), ("lz4", "mixed", 70000, 3),
        ("zstd", "xor16", 1024, 5), ("lz4", "random", 37, 4)]
# the autotuner's parse parameters: search strength and shortest match
TUNED = [("zstd", "mixed", 65536, 2, "strength=4", "mm=12"),
         ("zstd", "geom", 20000, 1, "strength=8", "mm=6"),
         ("zstd", "xor16", 40000, 1, "strength=5", "mm=6"),
         ("lz4", "xor16", 40000, 1, "strength=8", "mm=6"),
         ("lz4", "random", 70000, 1, "strength=4", "mm=5"),
         ("lz4", "halves", 70000, 2, "strength=7", "mm=5")]


def _key(codec, pattern, chunk, n, *extra):
    return (codec, str(chunk), str(n), pattern) + tuple(extra)


def _cases():
    """Every emulator run of this module (they are independent processes,
    run side by side by the `runs` fixture)."""
    keys = [_key(*c) for c in BIG]
    keys += [_key(c, p, ch, n) for c in ("lz4", "zstd")
             for p in ("zeros", "random", "ramp", "mixed", "xor16") for ch, n in CASES]
    keys += [_key(c, p, ch, n, "level=%d" % lv) for c, p, ch, n, lv in WIDE]
    keys += [_key(c, p, ch, n, "level=%d" % lv) for c, lv in (("lz4", 2), ("zstd", 3))
             for p in ("zeros", "mixed", "xor16") for ch, n in WIDE_SMALL]
    keys += [_key(c, p, ch, n, "refs", lv) for c, p, ch, n in REFS
             for lv in ("level=1", "level=3")]
    keys += [_key(c, p, ch, n, st, mm) for c, p, ch, n, st, mm in TUNED]
    return keys


@pytest.fixture(scope="module")
def runs(emu):
    from concurrent.futures import ThreadPoolExecutor

    def one(k):
        codec, chunk, n, pattern = k[:4]
        return k, subprocess.run([emu, codec, chunk, n, pattern, "7", *k[4:]],
                                 capture_output=True, text=True, timeout=900)

    with ThreadPoolExecutor(max_workers=max(1, os.cpu_count() or 1)) as ex:
        return dict(ex.map(one, _cases()))


def _run(runs, codec, pattern, chunk, n, *extra):
    r = runs[_key(codec, pattern, chunk, n, *extra)]
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.startswith("ok")


@pytest.mark.parametrize("codec,pattern,chunk,n", BIG)
def test_encoder_multi_block_chunks(runs, codec, pattern, chunk, n):
    _run(runs, codec, pattern, chunk, n)


@pytest.mark.parametrize("codec", ["lz4", "zstd"])
@pytest.mark.parametrize("pattern", ["zeros", "random", "ramp", "mixed", "xor16"])
@pytest.mark.parametrize("chunk,n", CASES)
def test_encoder_decodes_with_stock_library(runs, codec, pattern, chunk, n):
    _run(runs, codec, pattern, chunk, n)


@pytest.mark.parametrize("codec,pattern,chunk,n,level", WIDE)
def test_wide_window_levels(runs, codec, pattern, chunk, n, level):
    _run(runs, codec, pattern, chunk, n, "level=%d" % level)


@pytest.mark.parametrize("codec,level", [("lz4", 2), ("zstd", 3)])
@pytest.mark.parametrize("pattern", ["zeros", "mixed", "xor16"])
@pytest.mark.parametrize("chunk,n", WIDE_SMALL)
def test_wide_window_small_chunks(runs, codec, level, pattern, chunk, n):
    _run(runs, codec, pattern, chunk, n, "level=%d" % level)


@pytest.mark.parametrize("codec,pattern,chunk,n", REFS)
@pytest.mark.parametrize("level", ["level=1", "level=3"])
def test_encoder_per_chunk_references(runs, codec, pattern, chunk, n, level):
    """Chunks addressed through a per-chunk reference list (the shared
    encoder engine's batches) decode to their bytes."""
    _run(runs, codec, pattern, chunk, n, "refs", level)


@pytest.mark.parametrize("codec,pattern,chunk,n,strength,mm", TUNED)
def test_tuned_parse_parameters(runs, codec, pattern, chunk, n, strength, mm):
    """Chunks parsed with other search strengths and shortest matches (the
    autotuner's candidates) decode to their bytes."""
    _run(runs, codec, pattern, chunk, n, strength, mm)
