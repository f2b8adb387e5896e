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


def _run(emu, codec, pattern, chunk, n, *extra):
    r = subprocess.run([emu, codec, str(chunk), str(n), pattern, "7", *extra],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.startswith("ok")


@pytest.mark.parametrize("codec,pattern,chunk,n", BIG)
def test_encoder_multi_block_chunks(emu, codec, pattern, chunk, n):
    _run(emu, codec, pattern, chunk, n)


@pytest.mark.parametrize("codec", ["lz4", "zstd"])
@pytest.mark.parametrize("pattern", ["zeros", "random", "ramp", "mixed", "xor16"])
@pytest.mark.parametrize("chunk,n", CASES)
def test_encoder_decodes_with_stock_library(emu, codec, pattern, chunk, n):
    _run(emu, codec, pattern, chunk, n)


@pytest.mark.parametrize("codec,pattern,chunk,n", [("zstd", "mixed", 70000, 3),
                                                  ("lz4", "mixed", 70000, 3),
                                                  ("zstd", "xor16", 1024, 5),
                                                  ("lz4", "random", 37, 4)])
def test_encoder_per_chunk_references(emu, codec, pattern, chunk, n):
    """Chunks addressed through a per-chunk reference list (the shared
    encoder engine's batches) decode to their bytes."""
    _run(emu, codec, pattern, chunk, n, "refs")
