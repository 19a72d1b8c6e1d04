// Base64 decoding for the transcript wire format.
//
// HEAL's runtime writes every host tensor of a transcript as the base64 text
// (RFC 4648 section 4: standard alphabet, '=' padding) of its torch.save or
// np.save bytes and reads it back with base64.b64decode
// (python_execution/lattica_heal_runtime/serialization.py:27,31).  A server
// that takes its requests as transcripts decodes every request's payload on
// arrival, several MB for a large plaintext matrix, so this is host code on
// the request path: the text is cut into runs of whole 4-character groups
// and each run is decoded by its own thread into its own part of the output.
//
// Only the canonical encoding is accepted: a length that is a multiple of 4,
// every character in the alphabet, and '=' only as the last one or two
// characters.  Anything else (line breaks, other characters that
// b64decode discards, missing padding) is reported, and the caller passes
// such text to a lenient decoder instead, so no input decodes differently.
#include <cstdint>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "heal_internal.h"
#include "../../include/heal_gb300.h"

namespace heal {
namespace {

constexpr uint8_t kBad = 0xFF;

struct B64Table {
  uint8_t v[256];
  B64Table() {
    memset(v, kBad, sizeof v);
    for (int i = 0; i < 26; ++i) {
      v['A' + i] = (uint8_t)i;
      v['a' + i] = (uint8_t)(26 + i);
    }
    for (int i = 0; i < 10; ++i) v['0' + i] = (uint8_t)(52 + i);
    v['+'] = 62;
    v['/'] = 63;
  }
};
const B64Table kTable;

// Decodes `groups` full 4-character groups (no padding) from src into dst
// (3 bytes per group); false if a character is outside the alphabet.
bool decode_groups(const unsigned char *src, size_t groups, unsigned char *dst) {
  const uint8_t *t = kTable.v;
  uint32_t bad = 0;
  for (size_t g = 0; g < groups; ++g, src += 4, dst += 3) {
    const uint32_t a = t[src[0]], b = t[src[1]], c = t[src[2]], d = t[src[3]];
    bad |= a | b | c | d;
    const uint32_t w = (a << 18) | (b << 12) | (c << 6) | d;
    dst[0] = (unsigned char)(w >> 16);
    dst[1] = (unsigned char)(w >> 8);
    dst[2] = (unsigned char)w;
  }
  return (bad & 0xC0u) == 0;   // every valid value is below 64
}

}  // namespace
}  // namespace heal

using namespace heal;

extern "C" int heal_base64_decode(const char *src, size_t len, void *dst, size_t cap, size_t *written,
                                  int threads) {
  if (!written || (len && (!src || !dst)))
    return set_error(HEAL_ERR_INVALID_ARGUMENT, "heal_base64_decode: null pointer");
  *written = 0;
  if (len % 4) return set_error(HEAL_ERR_INVALID_ARGUMENT, "heal_base64_decode: length is not a multiple of 4");
  if (len == 0) return HEAL_OK;
  const unsigned char *s = (const unsigned char *)src;
  const size_t pad = s[len - 1] == '=' ? (s[len - 2] == '=' ? 2 : 1) : 0;
  const size_t out = len / 4 * 3 - pad;
  if (out > cap) return set_error(HEAL_ERR_INVALID_ARGUMENT, "heal_base64_decode: output buffer too small");
  unsigned char *d = (unsigned char *)dst;
  const size_t body = len / 4 - (pad ? 1 : 0);  // groups without padding

  // runs of at least 64 K groups (256 KB of text) per thread
  unsigned hw = std::thread::hardware_concurrency();
  size_t nt = threads > 0 ? (size_t)threads : (hw ? hw : 1);
  if (nt > 16) nt = 16;
  const size_t min_run = (size_t)1 << 16;
  if (nt > body / min_run) nt = body / min_run ? body / min_run : 1;

  bool ok = true;
  if (nt <= 1) {
    ok = decode_groups(s, body, d);
  } else {
    std::vector<std::thread> pool;
    std::vector<char> part_ok(nt, 1);
    const size_t per = (body + nt - 1) / nt;
    auto run = [&](size_t t) {
      const size_t g0 = t * per, g1 = g0 + per < body ? g0 + per : body;
      if (g0 < g1) part_ok[t] = decode_groups(s + 4 * g0, g1 - g0, d + 3 * g0);
    };
    size_t started = 1;  // runs 1 .. started-1 have their own thread
    try {
      for (size_t t = 1; t < nt; ++t) {
        pool.emplace_back(run, t);
        started = t + 1;
      }
    } catch (...) {
      // a thread could not be started: the calling thread takes its runs
    }
    run(0);
    for (size_t t = started; t < nt; ++t) run(t);
    for (auto &th : pool) th.join();
    for (char v : part_ok) ok = ok && v;
  }
  if (ok && pad) {
    // the last group: "xx==" (one byte) or "xxx=" (two bytes)
    const unsigned char *g = s + 4 * body;
    const uint8_t *t = kTable.v;
    const uint32_t a = t[g[0]], b = t[g[1]], c = pad == 1 ? t[g[2]] : 0;
    if ((a | b | c) & 0xC0u) {
      ok = false;
    } else {
      const uint32_t w = (a << 18) | (b << 12) | (c << 6);
      d[3 * body] = (unsigned char)(w >> 16);
      if (pad == 1) d[3 * body + 1] = (unsigned char)(w >> 8);
    }
  }
  if (!ok) return set_error(HEAL_ERR_INVALID_ARGUMENT, "heal_base64_decode: not canonical base64 text");
  *written = out;
  return HEAL_OK;
}
