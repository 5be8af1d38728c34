// Host-side decoders for compressed movie files (MRCZ: MRC slices stored as
// blosc chunks; zorro.loadData reads .mrcz through mrcz, zorro.py:3414).
//
// zr_lz4_decompress decodes one LZ4 block (the LZ4 and LZ4HC codecs of
// blosc) as the LZ4 block format describes it: a run of sequences, each a
// token byte (high nibble: literal count, low nibble: match length - 4; 15
// in either means more length bytes follow, added until one is below 255),
// the literals, then a 2-byte little-endian match offset and the match
// length bytes; the last sequence ends after its literals.  Every read and
// write is bounds-checked; malformed input returns -1 instead of touching
// memory outside the buffers.
#include <stddef.h>
#include <stdint.h>

#include "internal.h"
#include "zorro_gb300.h"

extern "C" long long zr_lz4_decompress(const void* src, size_t src_bytes, void* dst, size_t dst_bytes) {
  if (!src || !dst) return zr::set_error(ZR_EINVAL, "zr_lz4_decompress: null argument");
  const uint8_t* ip = (const uint8_t*)src;
  const uint8_t* const iend = ip + src_bytes;
  uint8_t* op = (uint8_t*)dst;
  uint8_t* const ostart = op;
  uint8_t* const oend = op + dst_bytes;
  while (ip < iend) {
    const unsigned token = *ip++;
    size_t lit = token >> 4;
    if (lit == 15) {
      unsigned b;
      do {
        if (ip >= iend) return zr::set_error(-1, "zr_lz4_decompress: truncated literal length");
        b = *ip++;
        lit += b;
      } while (b == 255);
    }
    if ((size_t)(iend - ip) < lit || (size_t)(oend - op) < lit)
      return zr::set_error(-1, "zr_lz4_decompress: literals overrun the buffers");
    for (size_t i = 0; i < lit; i++) op[i] = ip[i];
    ip += lit;
    op += lit;
    if (ip >= iend) break;  // the last sequence: literals only
    if (iend - ip < 2) return zr::set_error(-1, "zr_lz4_decompress: truncated match offset");
    const size_t off = (size_t)ip[0] | ((size_t)ip[1] << 8);
    ip += 2;
    size_t mlen = token & 15u;
    if (mlen == 15) {
      unsigned b;
      do {
        if (ip >= iend) return zr::set_error(-1, "zr_lz4_decompress: truncated match length");
        b = *ip++;
        mlen += b;
      } while (b == 255);
    }
    mlen += 4;
    if (off == 0 || off > (size_t)(op - ostart)) return zr::set_error(-1, "zr_lz4_decompress: bad match offset");
    if ((size_t)(oend - op) < mlen) return zr::set_error(-1, "zr_lz4_decompress: match overruns the output");
    const uint8_t* ref = op - off;
    for (size_t i = 0; i < mlen; i++) op[i] = ref[i];  // byte by byte: a match may overlap its own output
    op += mlen;
  }
  return (long long)(op - ostart);
}
