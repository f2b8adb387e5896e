// Runs the LZ4 and zstd encoder kernels under the CPU SIMT emulation and
// decodes every chunk with the stock liblz4 / libzstd -- TEST
// INFRASTRUCTURE ONLY.  Built with AddressSanitizer + UBSan (alignment) when
// available, so out-of-bounds and misaligned accesses abort with a report.
//
// usage: codec_emu <lz4|zstd> <chunk_bytes> <n_chunks> <pattern> <seed>
//                  [refs] [level=<n>] [strength=<n>] [mm=<n>]
#include "simt.hpp"

#include "../../chucky_gb300/csrc/lz4.cu"
#include "../../chucky_gb300/csrc/lz4_decode.cu"
#include "../../chucky_gb300/csrc/zstd.cu"
#include "../../chucky_gb300/csrc/zstd_decode.cu"

#include <dlfcn.h>
#include <string>

using namespace chucky;

namespace chucky {
void note_launches(unsigned) {}
} // namespace chucky

static uint64_t rng_state;
static uint64_t f_of(int t, uint64_t nf) { return uint64_t(t) % nf; }
static uint64_t rnd()
{
  uint64_t z = (rng_state += 0x9e3779b97f4a7c15ULL);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
  return z ^ (z >> 31);
}

static void fill(uint8_t* p, size_t n, const std::string& pat, size_t chunk)
{
  if (pat.rfind("file:", 0) == 0) { // repeat the file's bytes
    FILE* f = std::fopen(pat.c_str() + 5, "rb");
    std::vector<uint8_t> d;
    if (f) {
      uint8_t buf[65536];
      size_t k;
      while ((k = std::fread(buf, 1, sizeof buf, f)) > 0)
        d.insert(d.end(), buf, buf + k);
      std::fclose(f);
    }
    for (size_t i = 0; i < n; ++i)
      p[i] = d.empty() ? 0 : d[i % d.size()];
    return;
  }
  for (size_t i = 0; i < n; ++i) {
    if (pat == "zeros")
      p[i] = 0;
    else if (pat == "random")
      p[i] = uint8_t(rnd());
    else if (pat == "u200") // values 0..199: an even count of explicit weights
      p[i] = uint8_t(rnd() % 200);
    else if (pat == "u201") // values 0..200: an odd count
      p[i] = uint8_t(rnd() % 201);
    else if (pat == "geom") { // skewed: P(k) ~ 2^-(k+1), rare other bytes
      const uint64_t r = rnd();
      p[i] = (r & 511) == 0 ? uint8_t(r >> 9) : uint8_t(__builtin_ctzll(r | (1ull << 40)));
    } else if (pat == "halves") // random first half of each chunk, zeros after
      p[i] = (i % chunk) < chunk / 2 ? uint8_t(rnd()) : 0;
    else if (pat == "ramp")
      p[i] = uint8_t(i % 251);
    else if (pat == "xor16") { // u16 (x^y^z)*257 + noise(0..15)
      const size_t e = i / 2, x = e % 64, y = (e / 64) % 64, z = e / 4096;
      const uint16_t v = uint16_t(((x ^ y ^ z) * 257 + (rnd() & 15)));
      p[i] = (i & 1) ? uint8_t(v >> 8) : uint8_t(v);
    } else { // mixed: per-chunk classes
      const size_t c = i / chunk;
      const uint64_t h = (c * 0x9E3779B97F4A7C15ULL) >> 60;
      if (h < 8)
        p[i] = 0;
      else if (h < 12)
        p[i] = uint8_t(c * 37);
      else if (h < 14)
        p[i] = uint8_t(rnd() & 7);
      else
        p[i] = uint8_t(rnd());
    }
  }
}

int main(int argc, char** argv)
{
  if (argc < 6) {
    std::fprintf(stderr, "usage: codec_emu codec chunk_bytes n_chunks pattern seed\n");
    return 2;
  }
  {
    // slot runs of a partial batch (CodecBatch::id): entries 0-3 from slot
    // 10, 4-5 from slot 40, 6-8 from slot 7; waves start at id_base
    CodecBatch r{};
    r.n_runs = 3;
    const uint32_t first[4] = { 0, 4, 6, 9 }, slot[3] = { 10, 40, 7 };
    for (int k = 0; k < 4; ++k)
      r.run_first[k] = first[k];
    for (int k = 0; k < 3; ++k)
      r.run_slot[k] = slot[k];
    const uint64_t want[9] = { 10, 11, 12, 13, 40, 41, 7, 8, 9 };
    for (uint64_t base = 0; base < 9; ++base) {
      r.id_base = base;
      for (uint64_t i = 0; base + i < 9; ++i)
        if (r.id(i) != want[base + i]) {
          std::fprintf(stderr, "run mapping: entry %llu -> %llu\n",
                       (unsigned long long)(base + i), (unsigned long long)r.id(i));
          return 1;
        }
    }
  }
  const std::string codec = argv[1];
  const uint32_t chunk = uint32_t(std::stoul(argv[2]));
  const uint64_t n = std::stoull(argv[3]);
  const std::string pat = argv[4];
  rng_state = std::stoull(argv[5]);
  bool refs_mode = false;
  int level = 1, strength = 0, min_match = 0;
  for (int a = 6; a < argc; ++a) {
    const std::string opt = argv[a];
    if (opt == "refs")
      refs_mode = true;
    else if (opt.rfind("level=", 0) == 0)
      level = std::stoi(opt.substr(6));
    else if (opt.rfind("strength=", 0) == 0)
      strength = std::stoi(opt.substr(9));
    else if (opt.rfind("mm=", 0) == 0)
      min_match = std::stoi(opt.substr(3));
  }
  const uint64_t in_stride = (chunk + 255) / 256 * 256;
  const uint64_t bound = codec == "zstd"
                           ? chunk + (chunk >> 8) + (chunk < (128u << 10) ? ((128u << 10) - chunk) >> 11 : 0)
                           : chunk + chunk / 255 + 16;
  const uint64_t out_stride = (bound + 15) / 16 * 16;
  std::vector<uint8_t> in(n * in_stride + 256), out(n * out_stride + 64);
  std::vector<uint64_t> sizes(n);
  std::vector<uint8_t> flat(n * chunk);
  fill(flat.data(), flat.size(), pat, chunk);
  for (uint64_t c = 0; c < n; ++c)
    std::memcpy(in.data() + c * in_stride, flat.data() + c * chunk, chunk);
  CodecBatch b{};
  b.in = in.data();
  b.in_stride = in_stride;
  b.chunk_bytes = chunk;
  b.n_chunks = n;
  b.out = out.data();
  b.out_stride = out_stride;
  b.out_sizes = sizes.data();
  b.level = level;
  b.strength = strength;
  b.min_match = min_match;
  const size_t sb = codec == "zstd" ? zstd_scratch_bytes(n, chunk, level)
                                    : lz4_scratch_bytes(n, chunk, level);
  std::vector<uint8_t> scratch(sb);
  const cudaError_t e = codec == "zstd" ? launch_zstd(b, scratch.data(), nullptr)
                                        : launch_lz4(b, scratch.data(), nullptr);
  if (e != cudaSuccess) {
    std::fprintf(stderr, "launch failed %d\n", e);
    return 1;
  }
  void* zl = dlopen("libzstd.so.1", RTLD_NOW);
  void* ll = dlopen("liblz4.so.1", RTLD_NOW);
  auto zd = (size_t(*)(void*, size_t, const void*, size_t))(zl ? dlsym(zl, "ZSTD_decompress") : nullptr);
  auto ze = (unsigned (*)(size_t))(zl ? dlsym(zl, "ZSTD_isError") : nullptr);
  auto zn = (const char* (*)(size_t))(zl ? dlsym(zl, "ZSTD_getErrorName") : nullptr);
  auto ld = (int (*)(const char*, char*, int, int))(ll ? dlsym(ll, "LZ4_decompress_safe") : nullptr);
  if (!zd || !ld) {
    std::fprintf(stderr, "stock codecs missing\n");
    return 3;
  }
  uint64_t comp = 0;
  std::vector<uint8_t> dec(chunk + 64);
  for (uint64_t c = 0; c < n; ++c) {
    const uint8_t* src = out.data() + c * out_stride;
    if (sizes[c] > bound) {
      std::fprintf(stderr, "chunk %llu: size %llu above bound %llu\n",
                   (unsigned long long)c, (unsigned long long)sizes[c],
                   (unsigned long long)bound);
      return 1;
    }
    size_t got;
    if (codec == "zstd") {
      got = zd(dec.data(), dec.size(), src, sizes[c]);
      if (ze(got)) {
        std::fprintf(stderr, "chunk %llu: zstd error %s\n", (unsigned long long)c, zn(got));
        return 1;
      }
    } else {
      const int r = ld((const char*)src, (char*)dec.data(), int(sizes[c]), int(chunk));
      if (r < 0) {
        std::fprintf(stderr, "chunk %llu: lz4 error %d\n", (unsigned long long)c, r);
        return 1;
      }
      got = size_t(r);
    }
    if (got != chunk || std::memcmp(dec.data(), flat.data() + c * chunk, chunk)) {
      size_t at = 0;
      while (at < chunk && dec[at] == flat[c * chunk + at])
        ++at;
      std::fprintf(stderr, "chunk %llu: decoded bytes differ (got %zu, first at %zu: %u vs %u)\n",
                   (unsigned long long)c, got, at, unsigned(dec[at]),
                   unsigned(flat[c * chunk + at]));
      return 1;
    }
    comp += sizes[c];
  }
  if (codec == "zstd") {
    // the device decoder on the same frames, and on libzstd's frames of the
    // same chunks at levels 1, 3 and 19: every chunk back exactly
    auto zc = (size_t(*)(void*, size_t, const void*, size_t, int))dlsym(zl, "ZSTD_compress");
    auto zb = (size_t(*)(size_t))dlsym(zl, "ZSTD_compressBound");
    if (!zc || !zb)
      return 3;
    std::vector<uint8_t> frames;
    std::vector<uint64_t> offs, lens;
    for (uint64_t c = 0; c < n; ++c) { // ours
      offs.push_back(frames.size());
      lens.push_back(sizes[c]);
      frames.insert(frames.end(), out.data() + c * out_stride,
                    out.data() + c * out_stride + sizes[c]);
    }
    for (int lvl : { 1, 3, 19 })
      for (uint64_t c = 0; c < n; ++c) {
        std::vector<uint8_t> tmp(zb(chunk));
        const size_t k = zc(tmp.data(), tmp.size(), flat.data() + c * chunk, chunk, lvl);
        if (ze(k))
          return 1;
        offs.push_back(frames.size());
        lens.push_back(k);
        frames.insert(frames.end(), tmp.data(), tmp.data() + k);
      }
    const uint64_t nf = offs.size();
    std::vector<uint8_t> back(nf * in_stride, 0xAB);
    std::vector<uint32_t> st(nf, 99);
    if (launch_zstd_decode(frames.data(), offs.data(), lens.data(), nf, back.data(),
                           in_stride, chunk, st.data(), nullptr) != cudaSuccess)
      return 1;
    for (uint64_t f = 0; f < nf; ++f) {
      const uint64_t c = f % n;
      if (st[f] != 0 || std::memcmp(back.data() + f * in_stride, flat.data() + c * chunk, chunk)) {
        size_t at = 0;
        while (at < chunk && back[f * in_stride + at] == flat[c * chunk + at])
          ++at;
        std::fprintf(stderr, "frame %llu (%s): device zstd decoder status %u, first diff at %zu\n",
                     (unsigned long long)f, f < n ? "ours" : "libzstd", st[f], at);
        return 1;
      }
    }
    // malformed frames (cut short, garbage, bytes flipped) report an error
    // and stay in bounds (AddressSanitizer watches every access)
    std::vector<uint8_t> junk(4096 + lens[0]);
    for (auto& x : junk)
      x = uint8_t(rnd());
    std::vector<std::vector<uint8_t>> bad;
    for (uint64_t cut : { uint64_t(1), uint64_t(5), lens[0] / 2, lens[0] - 1 })
      if (cut < lens[0])
        bad.emplace_back(frames.begin() + offs[0], frames.begin() + offs[0] + cut);
    bad.push_back(junk);
    for (int t = 0; t < 64; ++t) {
      std::vector<uint8_t> b(frames.begin() + offs[f_of(t, nf)], frames.begin() + offs[f_of(t, nf)] + lens[f_of(t, nf)]);
      b[rnd() % b.size()] ^= uint8_t(1 + rnd() % 255);
      bad.push_back(b);
    }
    for (size_t t = 0; t < bad.size(); ++t) {
      uint64_t o = 0, l = bad[t].size();
      uint32_t s = 99;
      std::vector<uint8_t> tmp(chunk);
      if (launch_zstd_decode(bad[t].data(), &o, &l, 1, tmp.data(), chunk, chunk, &s, nullptr) !=
          cudaSuccess)
        return 1;
      if (s > 5) {
        std::fprintf(stderr, "malformed frame %zu: status %u\n", t, s);
        return 1;
      }
      if (t < 5 && s == 0) {
        std::fprintf(stderr, "malformed frame %zu decoded as valid\n", t);
        return 1;
      }
    }
  }
  if (codec == "lz4") {
    // the device decoder on the same blocks: every chunk back exactly
    std::vector<uint64_t> offs(n), lens(n);
    for (uint64_t c = 0; c < n; ++c) {
      offs[c] = c * out_stride;
      lens[c] = sizes[c];
    }
    std::vector<uint8_t> back(n * in_stride, 0xAB);
    std::vector<uint32_t> st(n, 99);
    if (launch_lz4_decode(out.data(), offs.data(), lens.data(), n, back.data(), in_stride,
                          chunk, st.data(), nullptr) != cudaSuccess)
      return 1;
    for (uint64_t c = 0; c < n; ++c)
      if (st[c] != 0 || std::memcmp(back.data() + c * in_stride, flat.data() + c * chunk, chunk)) {
        std::fprintf(stderr, "chunk %llu: device decoder status %u or bytes differ\n",
                     (unsigned long long)c, st[c]);
        return 1;
      }
    // malformed blocks (cut short, garbage) report an error and stay in
    // bounds (AddressSanitizer watches every access)
    std::vector<uint8_t> junk(out_stride * 2);
    for (auto& x : junk)
      x = uint8_t(rnd());
    const uint64_t cut = sizes[0] > 1 ? sizes[0] - 1 : 0;
    std::vector<uint8_t> bad(cut + 1);
    std::memcpy(bad.data(), out.data(), cut);
    const uint8_t* blocks[3] = { bad.data(), junk.data(), junk.data() + 7 };
    const uint64_t blens[3] = { cut, out_stride, out_stride - 7 };
    for (int t = 0; t < 3; ++t) {
      uint64_t o = 0, l = blens[t];
      uint32_t s = 99;
      std::vector<uint8_t> tmp(chunk);
      if (launch_lz4_decode(blocks[t], &o, &l, 1, tmp.data(), chunk, chunk, &s, nullptr) !=
          cudaSuccess)
        return 1;
      if (s == 0 && !(t == 0 && cut == sizes[0])) {
        std::fprintf(stderr, "malformed block %d decoded as valid\n", t);
        return 1;
      }
    }
  }
  if (refs_mode) {
    // The same chunks addressed one by one (CodecBatch::refs, as the shared
    // encoder engine gathers several streams' chunks): chunks in reverse
    // order in a buffer of another stride, outputs and sizes in reverse
    // slots of other buffers.  Every chunk must decode to its bytes.  (The
    // bytes themselves may differ from the first run here: the emulation
    // resolves stores of several lanes to one hash slot in thread order,
    // which varies from run to run; the GPU keeps one lane's store.)
    const uint64_t st2 = in_stride + 64, os2 = out_stride + 32;
    std::vector<uint8_t> in2(n * st2 + 256), out2(n * os2 + 64);
    std::vector<uint64_t> sizes2(n, 0);
    std::vector<ChunkRef> refs(n);
    for (uint64_t c = 0; c < n; ++c) {
      const uint64_t r = n - 1 - c;
      std::memcpy(in2.data() + r * st2, flat.data() + c * chunk, chunk);
      refs[c].in = in2.data() + r * st2;
      refs[c].out = out2.data() + r * os2;
      refs[c].size = sizes2.data() + r;
    }
    CodecBatch rb{};
    rb.chunk_bytes = chunk;
    rb.n_chunks = n;
    rb.level = level;
    rb.strength = strength;
    rb.min_match = min_match;
    rb.refs = refs.data();
    std::vector<uint8_t> scratch2(sb, 0x5A);
    if ((codec == "zstd" ? launch_zstd(rb, scratch2.data(), nullptr)
                         : launch_lz4(rb, scratch2.data(), nullptr)) != cudaSuccess)
      return 1;
    for (uint64_t c = 0; c < n; ++c) {
      const uint64_t r = n - 1 - c;
      const uint8_t* src = out2.data() + r * os2;
      size_t got = 0;
      if (codec == "zstd") {
        got = zd(dec.data(), dec.size(), src, sizes2[r]);
        if (ze(got))
          got = 0;
      } else {
        const int k = ld((const char*)src, (char*)dec.data(), int(sizes2[r]), int(chunk));
        got = k < 0 ? 0 : size_t(k);
      }
      if (sizes2[r] == 0 || sizes2[r] > bound || got != chunk ||
          std::memcmp(dec.data(), flat.data() + c * chunk, chunk)) {
        std::fprintf(stderr, "chunk %llu: refs addressing: size %llu, decoded %zu bytes\n",
                     (unsigned long long)c, (unsigned long long)sizes2[r], got);
        return 1;
      }
    }
  }
  std::printf("ok %s chunk=%u n=%llu pattern=%s level=%d ratio=%.3f\n", codec.c_str(), chunk,
              (unsigned long long)n, pat.c_str(), level, double(n * chunk) / double(comp));
  return 0;
}
