// OSKAR 2.6 visibility-file ingest.
//
// Host: the container index (64-byte file header, 20-byte chunk tags,
// optional names, payload, CRC-32C) and the small header/block tags are read
// and checked on the host.  Device: the large block payloads (cross-
// correlations and baseline u, v, w) are streamed by parallel host threads
// through pinned slots into one device array; their CRC-32C codes are
// computed on the GPU and the reshuffle [time][channel][baseline] ->
// [baseline][time][channel], the wavelength scaling and the u/v/w extrema
// run in one kernel.
//
// Reference (SKA-ScienceDataProcessor/RC): MS6/kernel/oskar/OskarBinReader.cpp
// mkFromFile :149-238 and readAndReshuffle :246-413, over the container
// library MS6/kernel/oskar/oskar_binary/src/ (index scan
// oskar_binary_create.c:48-282, lookup oskar_binary_query.c:38-68, payload
// read and CRC check oskar_binary_read.c:38-101, CRC-32C oskar_crc.c:45-160).
//
// Differences from the reference, all on inputs it does not handle:
//  * a block whose times or channels fall outside the header's counts, or
//    whose payloads are shorter than its own time count needs, is rejected
//    with GB_OSKAR_FORMAT_BAD (the reference writes or reads out of bounds);
//    so is max_times_per_block <= 0 (the reference divides by zero);
//  * a chunk whose block size is too small for its names and code is
//    GB_OSKAR_FILE_INVALID (the reference seeks backwards);
//  * every read starts its tag search at the first chunk, so readAndReshuffle
//    can be called again on the same VisData (the reference resumes the
//    search at its last block and fails with GB_OSKAR_TAG_NOT_FOUND);
//  * on an error the outputs' content is unspecified (the reference leaves
//    the blocks before the failing one written); the status is the one the
//    reference returns: the first failing step in block and tag order;
//  * an extreme that is zero keeps +0.0 for a maximum and -0.0 for a minimum
//    when both signs occur (the reference keeps the first zero it met).
#include <errno.h>
#include <fcntl.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <climits>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/rc_oskar.h"
#include "gb_common.cuh"
#include "gb_runtime.cuh"

namespace {

// --------------------------------------------------------------- CRC-32C
// Reflected Castagnoli polynomial; a finished code is re-opened by the final
// xor unless it equals the start value (the container's update rule).
constexpr uint32_t kPoly = 0x82F63B78u;
constexpr uint32_t kInit = 0xFFFFFFFFu;

struct CrcTables {
  uint32_t t[8][256];
  CrcTables() {
    for (uint32_t i = 0; i < 256; i++) {
      uint32_t c = i;
      for (int k = 0; k < 8; k++) c = (c >> 1) ^ (kPoly & (0u - (c & 1u)));
      t[0][i] = c;
    }
    for (int k = 1; k < 8; k++)
      for (int i = 0; i < 256; i++) t[k][i] = (t[k - 1][i] >> 8) ^ t[0][t[k - 1][i] & 0xFF];
  }
};

const CrcTables& crc_tables() {
  static const CrcTables T;
  return T;
}

uint32_t crc_register(uint32_t s, const uint8_t* p, size_t n) {
  const CrcTables& T = crc_tables();
  while (n >= 8) {
    const uint32_t lo = s ^ ((uint32_t)p[0] | (uint32_t)p[1] << 8 | (uint32_t)p[2] << 16 |
                             (uint32_t)p[3] << 24);
    const uint32_t hi =
        (uint32_t)p[4] | (uint32_t)p[5] << 8 | (uint32_t)p[6] << 16 | (uint32_t)p[7] << 24;
    s = T.t[7][lo & 0xFF] ^ T.t[6][(lo >> 8) & 0xFF] ^ T.t[5][(lo >> 16) & 0xFF] ^
        T.t[4][lo >> 24] ^ T.t[3][hi & 0xFF] ^ T.t[2][(hi >> 8) & 0xFF] ^
        T.t[1][(hi >> 16) & 0xFF] ^ T.t[0][hi >> 24];
    p += 8;
    n -= 8;
  }
  while (n--) s = (s >> 8) ^ T.t[0][(s ^ *p++) & 0xFF];
  return s;
}

uint32_t reopen(uint32_t code) { return code == kInit ? code : code ^ kInit; }

uint32_t crc_continue(uint32_t code, const void* p, size_t n) {
  return crc_register(reopen(code), (const uint8_t*)p, n) ^ kInit;
}

// The register after n zero bytes is a linear map of the register before
// them (GF(2) 32x32 matrix, stored by columns).  With it, the register over a
// message split into chunks is the xor of each chunk's register from zero
// carried over the bytes that follow the chunk.
struct Op {
  uint32_t c[32];
};

uint32_t op_apply(const Op& a, uint32_t v) {
  uint32_t r = 0;
  for (int b = 0; v; b++, v >>= 1)
    if (v & 1u) r ^= a.c[b];
  return r;
}

Op op_then(const Op& first, const Op& second) {  // second after first
  Op r;
  for (int j = 0; j < 32; j++) r.c[j] = op_apply(second, first.c[j]);
  return r;
}

Op op_identity() {
  Op r;
  for (int j = 0; j < 32; j++) r.c[j] = 1u << j;
  return r;
}

struct ZeroOps {  // pw[k]: 2^k zero bytes
  Op pw[64];
  ZeroOps() {
    const CrcTables& T = crc_tables();
    for (int b = 0; b < 32; b++) {
      const uint32_t s = 1u << b;
      pw[0].c[b] = (s >> 8) ^ T.t[0][s & 0xFF];
    }
    for (int k = 1; k < 64; k++) pw[k] = op_then(pw[k - 1], pw[k - 1]);
  }
};

const ZeroOps& zero_ops() {
  static const ZeroOps Z;
  return Z;
}

uint32_t zeros_apply(uint64_t n, uint32_t v) {
  const ZeroOps& Z = zero_ops();
  for (int k = 0; n; k++, n >>= 1)
    if (n & 1u) v = op_apply(Z.pw[k], v);
  return v;
}

Op zeros_op(uint64_t n) {
  const ZeroOps& Z = zero_ops();
  Op r = op_identity();
  for (int k = 0; n; k++, n >>= 1)
    if (n & 1u) r = op_then(r, Z.pw[k]);
  return r;
}

constexpr int kCrcChunkLog = 12;  // 4 KiB per thread
constexpr int64_t kCrcChunk = int64_t(1) << kCrcChunkLog;
constexpr int kCrcPowers = 28;  // chunk counts below 2^28 (1 TiB payloads)

struct CrcJob {
  int64_t off;          // byte offset of the payload in the device array (16-aligned)
  int64_t n;            // payload bytes
  int64_t first_chunk;  // global index of its first chunk
  uint32_t last[32];    // zero-byte map over the last chunk's length
};

// ---------------------------------------------------------------- container
enum : int { T_CHAR = 0x01, T_INT = 0x02, T_SINGLE = 0x04, T_DOUBLE = 0x08,
             T_COMPLEX = 0x20, T_MATRIX = 0x40 };
enum : int { G_HEADER = 11, G_BLOCK = 12 };
// OskarBinReader.cpp:67-100
enum : int { H_NUM_TAGS_PER_BLOCK = 2, H_AMP_TYPE = 4, H_MAX_TIMES_PER_BLOCK = 5,
             H_NUM_TIMES_TOTAL = 6, H_NUM_CHANNELS = 7, H_NUM_STATIONS = 8,
             H_FREQ_START_HZ = 9, H_FREQ_INC_HZ = 10, H_CHANNEL_BW_HZ = 11,
             H_TIME_START_MJD = 12, H_TIME_INC_SEC = 13, H_TIME_AVERAGE_SEC = 14,
             H_PHASE_CENTRE = 15, H_TELESCOPE_CENTRE = 16 };
enum : int { B_DIM_START_AND_SIZE = 1, B_FREQ_REF_INC_HZ = 2, B_TIME_REF_INC_MJD = 3,
             B_CROSS_CORR = 5, B_UU = 6, B_VV = 7, B_WW = 8 };

struct Chunk {
  int type = 0, group = 0, tag = 0;
  bool ext = false;
  int32_t user = 0;
  int64_t off = 0, size = 0;
  uint32_t crc = 0, crc_hdr = 0;
  std::string gname, tname;
};

int32_t le32(const uint8_t* p) {
  return (int32_t)((uint32_t)p[0] | (uint32_t)p[1] << 8 | (uint32_t)p[2] << 16 |
                   (uint32_t)p[3] << 24);
}

int64_t le64(const uint8_t* p) {
  uint64_t v = 0;
  for (int i = 7; i >= 0; i--) v = v << 8 | p[i];
  return (int64_t)v;
}

bool pread_full(int fd, void* dst, size_t n, int64_t off) {
  uint8_t* p = (uint8_t*)dst;
  while (n) {
    const size_t want = n > (size_t(1) << 30) ? (size_t(1) << 30) : n;
    const ssize_t r = pread(fd, p, want, (off_t)off);
    if (r < 0) {
      if (errno == EINTR) continue;
      return false;
    }
    if (r == 0) return false;
    p += r;
    n -= (size_t)r;
    off += r;
  }
  return true;
}

int fail(int code, const char* fmt, const char* what) {
  gb_set_error(code, fmt, what);
  return code;
}

}  // namespace

struct oskar_Binary {
  int fd = -1;
  int64_t file_size = 0;
  std::vector<Chunk> chunks;
  ~oskar_Binary() {
    if (fd >= 0) close(fd);
  }
};

namespace {

int bin_open(const char* path, oskar_Binary** out) {
  *out = nullptr;
  const int fd = open(path, O_RDONLY | O_CLOEXEC);
  if (fd < 0) return fail(GB_OSKAR_OPEN_FAIL, "cannot open %s", path);
  oskar_Binary* b = new oskar_Binary;
  b->fd = fd;
  struct stat sb;
  if (fstat(fd, &sb) != 0) {
    delete b;
    return fail(GB_OSKAR_READ_FAIL, "cannot stat %s", path);
  }
  b->file_size = (int64_t)sb.st_size;
  uint8_t hdr[64];
  if (!pread_full(fd, hdr, 64, 0)) {
    delete b;
    return fail(GB_OSKAR_READ_FAIL, "%s: no 64-byte file header", path);
  }
  if (memcmp(hdr, "OSKARBIN", 8) != 0) {
    delete b;
    return fail(GB_OSKAR_FILE_INVALID, "%s: not an OSKAR binary file", path);
  }
  const int version = (int8_t)hdr[9];
  if (version > 2) {
    delete b;
    return fail(GB_OSKAR_VERSION_UNKNOWN, "%s: unknown format version", path);
  }
  int status = 0;
  if (version == 1) {  // version-1 files record the writer's byte order and sizes
    if (hdr[10] != 0) {
      delete b;
      return fail(GB_OSKAR_ENDIAN_MISMATCH, "%s: big-endian data", path);
    }
    if (hdr[12] != 4) status = GB_OSKAR_INT_UNKNOWN;
    if (hdr[14] != 4) status = GB_OSKAR_FLOAT_UNKNOWN;
    if (hdr[15] != 8) status = GB_OSKAR_DOUBLE_UNKNOWN;
    if (status) {
      delete b;
      return fail(status, "%s: incompatible type sizes", path);
    }
  }
  int64_t pos = 64;
  for (;;) {
    uint8_t t[20];
    if (pos + 20 > b->file_size || !pread_full(fd, t, 20, pos)) break;
    if (t[0] != 'T' || t[2] != 'G' || (t[4] & 0x1F) != 0) {
      status = GB_OSKAR_FILE_INVALID;
      break;
    }
    const int fv = (int)(int8_t)t[1] - 0x40;
    if (fv < 1 || fv > 2) {
      status = GB_OSKAR_VERSION_UNKNOWN;
      break;
    }
    if (fv > 1) {  // element size check; the scan goes on after a failure
      int es = (int8_t)t[3];
      const int ty = t[5];
      if (ty & T_MATRIX) es /= 4;
      if (ty & T_COMPLEX) es /= 2;
      if (ty & T_CHAR) {
        if (es != 1) status = GB_OSKAR_FORMAT_BAD;
      } else if (ty & T_INT) {
        if (es != 4) status = GB_OSKAR_INT_UNKNOWN;
      } else if (ty & T_SINGLE) {
        if (es != 4) status = GB_OSKAR_FLOAT_UNKNOWN;
      } else if (ty & T_DOUBLE) {
        if (es != 8) status = GB_OSKAR_DOUBLE_UNKNOWN;
      } else {
        status = GB_OSKAR_TYPE_UNKNOWN;
      }
    }
    Chunk c;
    c.type = t[5];
    c.group = t[6];
    c.tag = t[7];
    c.user = le32(t + 8);
    uint32_t crc = crc_continue(kInit, t, 20);
    c.size = le64(t + 12) - ((t[4] & 0x40) ? 4 : 0);
    pos += 20;
    if (t[4] & 0x80) {
      c.ext = true;
      c.size -= (int64_t)t[6] + t[7];
    }
    if (c.size < 0) {
      status = GB_OSKAR_FILE_INVALID;
      break;
    }
    if (c.ext) {
      // both names end in NUL; an empty name field is a failed read there
      char names[512];
      if (t[6] == 0 || t[7] == 0 || !pread_full(fd, names, (size_t)t[6] + t[7], pos)) {
        status = GB_OSKAR_FILE_INVALID;
        break;
      }
      crc = crc_continue(crc, names, t[6]);
      crc = crc_continue(crc, names + t[6], t[7]);
      c.gname.assign(names, strnlen(names, t[6]));
      c.tname.assign(names + t[6], strnlen(names + t[6], t[7]));
      pos += (int64_t)t[6] + t[7];
    }
    c.off = pos;
    c.crc_hdr = crc;
    pos += c.size;
    if (t[4] & 0x40) {
      uint8_t cb[4];
      if (pos + 4 > b->file_size || !pread_full(fd, cb, 4, pos)) {
        status = GB_OSKAR_FILE_INVALID;
        break;
      }
      c.crc = (uint32_t)le32(cb);
      pos += 4;
    }
    b->chunks.push_back(std::move(c));
  }
  if (status) {
    delete b;
    return fail(status, "%s: malformed chunk index", path);
  }
  *out = b;
  return 0;
}

int query(const oskar_Binary* b, int search, int type, int group, int tag, int user) {
  for (int i = search; i < (int)b->chunks.size(); i++) {
    const Chunk& c = b->chunks[i];
    if (!c.ext && c.type == type && c.group == group && c.tag == tag && c.user == user) return i;
  }
  return -1;
}

// Host read of a (small) payload with its CRC check.
int read_tag(const oskar_Binary* b, int search, int type, int group, int tag, int user,
             size_t cap, void* dst, size_t* got = nullptr) {
  if (got) *got = 0;
  const int i = query(b, search, type, group, tag, user);
  if (i < 0) {
    gb_set_error(GB_OSKAR_TAG_NOT_FOUND, "OSKAR tag (%d,%d,%d) not found", group, tag, user);
    return GB_OSKAR_TAG_NOT_FOUND;
  }
  const Chunk& c = b->chunks[i];
  if (c.size == 0) return 0;
  if (!dst || cap < (size_t)c.size) {
    gb_set_error(GB_OSKAR_MEMORY_NOT_ALLOCATED, "OSKAR tag (%d,%d,%d) larger than expected",
                 group, tag, user);
    return GB_OSKAR_MEMORY_NOT_ALLOCATED;
  }
  if (!pread_full(b->fd, dst, (size_t)c.size, c.off)) {
    gb_set_error(GB_OSKAR_READ_FAIL, "OSKAR tag (%d,%d,%d): short read", group, tag, user);
    return GB_OSKAR_READ_FAIL;
  }
  if (c.crc && crc_continue(c.crc_hdr, dst, (size_t)c.size) != c.crc) {
    gb_set_error(GB_OSKAR_CRC_FAIL, "OSKAR tag (%d,%d,%d): CRC mismatch", group, tag, user);
    return GB_OSKAR_CRC_FAIL;
  }
  if (got) *got = (size_t)c.size;
  return 0;
}

// ------------------------------------------------------------ device kernels
__device__ __forceinline__ unsigned long long order_key(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

// Extrema are kept as order keys and compared as 64-bit integers: this part's
// FP64 pipe is narrow, and a NaN (which never replaces a value in the
// reference's std::max / std::min) is recognised from its bits and mapped to
// the neutral key.
__device__ __forceinline__ bool is_nan_bits(double x) {
  return ((unsigned long long)__double_as_longlong(x) << 1) > 0xFFE0000000000000ull;
}
__device__ __forceinline__ unsigned long long key_for_max(double x) {
  return is_nan_bits(x) ? 0ull : order_key(x);
}
__device__ __forceinline__ unsigned long long key_for_min(double x) {
  return is_nan_bits(x) ? ~0ull : order_key(x);
}

double key_value(unsigned long long k) {
  const unsigned long long b = (k >> 63) ? (k & 0x7FFFFFFFFFFFFFFFull) : ~k;
  double x;
  memcpy(&x, &b, 8);
  return x;
}

unsigned long long host_key(double x) {
  unsigned long long b;
  memcpy(&b, &x, 8);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

__device__ __forceinline__ uint32_t dev_apply(const uint32_t* cols, uint32_t v) {
  uint32_t r = 0;
#pragma unroll
  for (int b = 0; b < 32; b++) r ^= (0u - ((v >> b) & 1u)) & cols[b];
  return r;
}

// Slicing-by-8 step over 8 bytes (two little-endian words).
__device__ __forceinline__ uint32_t crc_step8(const uint32_t (*tab)[256], uint32_t s, uint32_t lo,
                                              uint32_t hi) {
  const uint32_t a = s ^ lo;
  return tab[7][a & 0xFF] ^ tab[6][(a >> 8) & 0xFF] ^ tab[5][(a >> 16) & 0xFF] ^
         tab[4][a >> 24] ^ tab[3][hi & 0xFF] ^ tab[2][(hi >> 8) & 0xFF] ^
         tab[1][(hi >> 16) & 0xFF] ^ tab[0][hi >> 24];
}

__device__ __forceinline__ uint32_t crc_step16(const uint32_t (*tab)[256], uint32_t s,
                                               const uint4& x) {
  return crc_step8(tab, crc_step8(tab, s, x.x, x.y), x.z, x.w);
}

// Four threads per 4 KiB chunk, one per 1 KiB quarter: each runs the
// slicing-by-8 register from zero over its quarter and carries it to the
// chunk's end with the 3/2/1 KiB zero-byte map; two shuffles join the
// quarters; the first lane carries the chunk to its payload's end (binary
// powers of the whole-chunk map, then the last chunk's length) and the
// payload registers are xor-accumulated.  A payload's short last chunk is
// run by its first lane alone.  pw holds kCrcPowers maps for 2^j whole
// chunks, then the three quarter maps.
__global__ void __launch_bounds__(256) k_crc32c(const uint8_t* __restrict__ base,
                                                const CrcJob* __restrict__ jobs, int n_jobs,
                                                int64_t total_chunks,
                                                const uint32_t* __restrict__ pw,
                                                uint32_t* __restrict__ out) {
  __shared__ uint32_t tab[8][256];
  __shared__ uint32_t spw[kCrcPowers + 3][32];
  const int tid = threadIdx.x;
  {
    uint32_t c = (uint32_t)tid;
    for (int k = 0; k < 8; k++) c = (c >> 1) ^ (kPoly & (0u - (c & 1u)));
    tab[0][tid] = c;
  }
  __syncthreads();
  for (int k = 1; k < 8; k++) {
    tab[k][tid] = (tab[k - 1][tid] >> 8) ^ tab[0][tab[k - 1][tid] & 0xFF];
    __syncthreads();
  }
  for (int i = tid; i < (kCrcPowers + 3) * 32; i += blockDim.x) spw[i / 32][i % 32] = pw[i];
  __syncthreads();
  const int lane = tid & 31;
  constexpr int Q = (int)(kCrcChunk / 64);  // uint4 words per quarter
  const int64_t total = total_chunks * 4;
  // every lane of a warp runs the same iterations (shuffles and the xor scan
  // need the whole warp); lanes past the end carry job -1
  for (int64_t t0 = (int64_t)blockIdx.x * blockDim.x + (tid & ~31); t0 < total;
       t0 += (int64_t)gridDim.x * blockDim.x) {
    const int64_t gt = t0 + lane, g = gt >> 2;
    const int q = (int)(gt & 3);
    int lo = -1;
    uint32_t s = 0;
    int64_t i = 0, k = 0;
    if (gt < total) {
      int hi = n_jobs - 1;  // last job with first_chunk <= g
      lo = 0;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (jobs[mid].first_chunk <= g) lo = mid;
        else hi = mid - 1;
      }
      const CrcJob& J = jobs[lo];
      i = g - J.first_chunk;
      k = (J.n + kCrcChunk - 1) >> kCrcChunkLog;
      const int64_t len = (i == k - 1) ? J.n - i * kCrcChunk : kCrcChunk;
      const uint8_t* p = base + J.off + i * kCrcChunk;
      const uint4* w4 = reinterpret_cast<const uint4*>(p);
      if (len == kCrcChunk) {
        const uint4* qq = w4 + q * Q;
        uint32_t r = 0;
#pragma unroll 4
        for (int w = 0; w < Q; w++) r = crc_step16(tab, r, __ldg(qq + w));
        s = q < 3 ? dev_apply(spw[kCrcPowers + 2 - q], r) : r;
      } else if (q == 0) {
        const int64_t words = len >> 4;
        for (int64_t w = 0; w < words; w++) s = crc_step16(tab, s, __ldg(w4 + w));
        for (int64_t j = words << 4; j < len; j++) s = (s >> 8) ^ tab[0][(s ^ p[j]) & 0xFF];
      }
    }
    s ^= __shfl_xor_sync(0xFFFFFFFFu, s, 1);  // the four quarters of one chunk
    s ^= __shfl_xor_sync(0xFFFFFFFFu, s, 2);
    if (q != 0) s = 0;
    if (lo >= 0 && q == 0 && i < k - 1) {
      const int64_t m = k - 2 - i;  // whole chunks between this one and the last
      for (int j = 0; j < kCrcPowers; j++)
        if ((m >> j) & 1) s = dev_apply(spw[j], s);
      s = dev_apply(jobs[lo].last, s);
    }
    // Chunks of one payload are consecutive lanes: an inclusive xor scan within
    // each run of equal jobs leaves the run's total in its last lane, which
    // alone issues the atomic (same-address atomics serialise in L2).
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, s, o);
      const int tj = __shfl_up_sync(0xFFFFFFFFu, lo, o);
      if (lane >= o && tj == lo) s ^= t;
    }
    const int next = __shfl_down_sync(0xFFFFFFFFu, lo, 1);
    if (lo >= 0 && (lane == 31 || next != lo)) atomicXor(out + lo, s);
  }
}

// kCrcPowers maps for 2^j whole chunks, then the maps for 1, 2, 3 quarters.
std::vector<uint32_t> crc_device_maps() {
  std::vector<uint32_t> pw((kCrcPowers + 3) * 32);
  const ZeroOps& Z = zero_ops();
  for (int j = 0; j < kCrcPowers; j++) memcpy(&pw[j * 32], Z.pw[kCrcChunkLog + j].c, 128);
  for (int q = 1; q <= 3; q++)
    memcpy(&pw[(kCrcPowers + q - 1) * 32], zeros_op((uint64_t)q * (kCrcChunk / 4)).c, 128);
  return pw;
}

struct BlockDesc {
  int64_t amp, u, v, w;  // byte offsets of the block's payloads in the device array
  int32_t t0, nt;        // first time index, times in the block
  int32_t il;            // first of its num_channels 1/lambda values
  int32_t pad;
};

__global__ void k_oskar_init_extrema(unsigned long long* __restrict__ blw, int32_t nb,
                                     unsigned long long kmax, unsigned long long kmin) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nb) {
    blw[2 * i] = kmax;
    blw[2 * i + 1] = kmin;
  }
}

// Tiled transpose through shared memory, persistent: each CTA walks work
// items (block, channel, tile of 32 baselines).  For an item it walks the
// block's times in groups of 8: the group's amplitudes (8 x 32 points x 64 B,
// 2 KiB contiguous per time) and u,v,w (256 B contiguous per time and
// component) are read coalesced, then each warp writes one baseline's 8 times
// (512 B of amplitudes and 192 B of u,v,w contiguous for one channel).  The
// u/v/w extrema of a CTA go to its own slot of gm (6 keys; the host reduces
// the slots): same-address atomics from every CTA would serialise in L2.
constexpr int kRT = 8;   // times per group
constexpr int kRB = 32;  // baselines per tile

__global__ void __launch_bounds__(256, 4) k_oskar_reshuffle(
    const uint8_t* __restrict__ raw, const BlockDesc* __restrict__ blocks, int32_t n_blocks,
    const double* __restrict__ invl, int32_t nb, int32_t nc, int32_t T,
    double* __restrict__ amps, double* __restrict__ uvws, unsigned long long* __restrict__ gm,
    unsigned long long* __restrict__ blw) {
  // rows padded so the transposed reads are free of bank conflicts: one
  // baseline (64 B) per time row of amplitudes, one double per row of u,v,w
  __shared__ double2 sa[kRT][kRB + 1][4];
  __shared__ double su[3][kRT][kRB + 1];
  __shared__ unsigned long long red[6][8];
  const int tiles = (nb + kRB - 1) / kRB;
  const int64_t items = (int64_t)n_blocks * nc * tiles;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  unsigned long long mx[3] = {0ull, 0ull, 0ull}, mn[3] = {~0ull, ~0ull, ~0ull};
  for (int64_t item = blockIdx.x; item < items; item += gridDim.x) {
    const int blk = (int)(item / ((int64_t)nc * tiles));
    const int rem = (int)(item - (int64_t)blk * nc * tiles);
    const int c = rem / tiles;
    const int b0 = (rem - c * tiles) * kRB;
    const BlockDesc bd = blocks[blk];
    const double2* A = reinterpret_cast<const double2*>(raw + bd.amp);
    const double* UVW[3] = {reinterpret_cast<const double*>(raw + bd.u),
                            reinterpret_cast<const double*>(raw + bd.v),
                            reinterpret_cast<const double*>(raw + bd.w)};
    const double il = invl[bd.il + c];
    unsigned long long wmax[kRB / 8], wmin[kRB / 8];  // this warp's baselines
#pragma unroll
    for (int i = 0; i < kRB / 8; i++) {
      wmax[i] = 0ull;
      wmin[i] = ~0ull;
    }
    for (int g0 = 0; g0 < bd.nt; g0 += kRT) {
      const int gn = min(kRT, bd.nt - g0);
#pragma unroll
      for (int it = 0; it < kRT * kRB * 4 / 256; it++) {  // amplitudes, 16 B per thread
        const int e = it * 256 + tid, t = e / (kRB * 4), r = e - t * (kRB * 4);
        const int b = r >> 2, k = r & 3;
        if (t < gn && b0 + b < nb)
          sa[t][b][k] = __ldg(A + 4 * (((int64_t)(g0 + t) * nc + c) * nb + b0 + b) + k);
      }
      {
        const int t = tid / kRB, b = tid - t * kRB;  // 256 threads = 8 times x 32 baselines
        if (t < gn && b0 + b < nb) {
          const int64_t j = (int64_t)(g0 + t) * nb + b0 + b;
#pragma unroll
          for (int k = 0; k < 3; k++) su[k][t][b] = __ldg(UVW[k] + j) * il;
        }
      }
      __syncthreads();
#pragma unroll
      for (int it = 0; it < kRB / 8; it++) {
        const int b = it * 8 + warp;
        if (b0 + b < nb) {
          const int64_t row = (int64_t)T * (b0 + b) + bd.t0 + g0;  // point (b, first time)
          {
            const int t = lane >> 2, k = lane & 3;
            if (t < gn)
              reinterpret_cast<double2*>(amps)[4 * ((row + t) * nc + c) + k] = sa[t][b][k];
          }
          if (lane < 3 * kRT) {
            const int t = lane / 3, k = lane - 3 * t;
            if (t < gn) {
              const double x = su[k][t][b];
              uvws[3 * ((row + t) * nc + c) + k] = x;
              const unsigned long long kx = key_for_max(x), kn = key_for_min(x);
              // constant indices only: a lane-dependent index would put the
              // accumulators in local memory
#pragma unroll
              for (int q = 0; q < 3; q++)
                if (q == k) {
                  mx[q] = max(mx[q], kx);
                  mn[q] = min(mn[q], kn);
                }
              if (k == 2) {
                wmax[it] = max(wmax[it], kx);
                wmin[it] = min(wmin[it], kn);
              }
            }
          }
        }
      }
      __syncthreads();
    }
    // per-baseline w extrema: reduce over the warp, one atomic pair per baseline
#pragma unroll
    for (int it = 0; it < kRB / 8; it++) {
      unsigned long long a = wmax[it], m = wmin[it];
      for (int o = 16; o; o >>= 1) {
        a = max(a, __shfl_xor_sync(0xFFFFFFFFu, a, o));
        m = min(m, __shfl_xor_sync(0xFFFFFFFFu, m, o));
      }
      const int b = b0 + it * 8 + warp;
      if (lane == 0 && b < nb && bd.nt > 0) {
        atomicMax(blw + 2 * b, a);
        atomicMin(blw + 2 * b + 1, m);
      }
    }
  }
  // CTA reduction of the six global extrema into this CTA's slot
#pragma unroll
  for (int k = 0; k < 3; k++) {
    for (int o = 16; o; o >>= 1) {
      mx[k] = max(mx[k], __shfl_xor_sync(0xFFFFFFFFu, mx[k], o));
      mn[k] = min(mn[k], __shfl_xor_sync(0xFFFFFFFFu, mn[k], o));
    }
  }
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
      red[k][warp] = mx[k];
      red[3 + k][warp] = mn[k];
    }
  }
  __syncthreads();
  if (tid < 6) {
    unsigned long long r = red[tid][0];
    for (int i = 1; i < 8; i++) r = tid < 3 ? max(r, red[tid][i]) : min(r, red[tid][i]);
    gm[6 * (int64_t)blockIdx.x + tid] = r;
  }
}

__global__ void k_oskar_records(const double* __restrict__ amps,
                                const double* __restrict__ uvws, int32_t T, int32_t nc,
                                int32_t freq, int32_t pol, int64_t lo, int64_t n, int32_t ref_index,
                                double* __restrict__ out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = lo + i, bl = p / T, t = p - bl * T;
    const int64_t full = (bl * T + t) * nc + freq;
    const int64_t ui = ref_index ? 3 * (t + (int64_t)T * bl) : 3 * full;
    double* o = out + 5 * i;
    o[0] = uvws[ui];
    o[1] = uvws[ui + 1];
    o[2] = uvws[ui + 2];
    o[3] = amps[8 * full + 2 * pol];
    o[4] = amps[8 * full + 2 * pol + 1];
  }
}

template <typename VT>
__global__ void k_oskar_extract(const double* __restrict__ amps, const double* __restrict__ uvws,
                                int32_t nc, int32_t freq, int32_t pol, int64_t n,
                                double* __restrict__ uvw, VT* __restrict__ vis) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t full = i * nc + freq;
    uvw[3 * i] = uvws[3 * full];
    uvw[3 * i + 1] = uvws[3 * full + 1];
    uvw[3 * i + 2] = uvws[3 * full + 2];
    const double2 a = reinterpret_cast<const double2*>(amps)[4 * full + pol];
    if constexpr (sizeof(VT) == 8) vis[i] = make_float2((float)a.x, (float)a.y);
    else vis[i] = a;
  }
}

// ------------------------------------------------------------ host pipeline
constexpr int64_t kSlot = int64_t(8) << 20;  // pinned staging slot

// Grow-only pool of pinned slots shared by every reader thread of the process.
struct PinnedPool {
  std::mutex m;
  std::vector<void*> free_slots;
  void* get() {
    {
      std::lock_guard<std::mutex> g(m);
      if (!free_slots.empty()) {
        void* p = free_slots.back();
        free_slots.pop_back();
        return p;
      }
    }
    void* p = nullptr;
    if (cudaHostAlloc(&p, (size_t)kSlot, cudaHostAllocDefault) != cudaSuccess) return nullptr;
    return p;
  }
  void put(void* p) {
    if (!p) return;
    std::lock_guard<std::mutex> g(m);
    free_slots.push_back(p);
  }
};

PinnedPool& pinned_pool() {
  static PinnedPool* P = new PinnedPool;  // never destroyed: the slots live as long as the process
  return *P;
}

struct Piece {
  int64_t file_off, dev_off, len;
};

// Parallel pread -> pinned slot -> cudaMemcpyAsync of every piece; returns when
// all copies are complete.
int stream_pieces(int fd, const std::vector<Piece>& pieces, uint8_t* d_raw) {
  if (pieces.empty()) return 0;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return GB_ERR_CUDA;
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const int K = (int)std::min<size_t>(pieces.size(), std::min(16u, hw));
  std::atomic<size_t> next{0};
  std::atomic<int> err{0};
  auto worker = [&]() {
    if (cudaSetDevice(dev) != cudaSuccess) {
      err = GB_ERR_CUDA;
      return;
    }
    cudaStream_t st = nullptr;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    void* slot[2] = {pinned_pool().get(), pinned_pool().get()};
    bool used[2] = {false, false};
    if (!slot[0] || !slot[1] || cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) ||
        cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming) ||
        cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming)) {
      err = GB_ERR_NOMEM;
    } else {
      int use = 0;
      for (;;) {
        const size_t i = next.fetch_add(1);
        if (i >= pieces.size() || err.load()) break;
        const Piece& pc = pieces[i];
        if (used[use] && cudaEventSynchronize(ev[use]) != cudaSuccess) {
          err = GB_ERR_CUDA;
          break;
        }
        if (!pread_full(fd, slot[use], (size_t)pc.len, pc.file_off)) {
          err = GB_OSKAR_READ_FAIL;
          break;
        }
        if (cudaMemcpyAsync(d_raw + pc.dev_off, slot[use], (size_t)pc.len,
                            cudaMemcpyHostToDevice, st) != cudaSuccess ||
            cudaEventRecord(ev[use], st) != cudaSuccess) {
          err = GB_ERR_CUDA;
          break;
        }
        used[use] = true;
        use ^= 1;
      }
    }
    if (st && cudaStreamSynchronize(st) != cudaSuccess) err = GB_ERR_CUDA;
    for (int k = 0; k < 2; k++) {
      if (ev[k]) cudaEventDestroy(ev[k]);
      pinned_pool().put(slot[k]);
    }
    if (st) cudaStreamDestroy(st);
  };
  std::vector<std::thread> th;
  for (int k = 1; k < K; k++) th.emplace_back(worker);
  worker();
  for (auto& t : th) t.join();
  const int e = err.load();
  if (e == GB_OSKAR_READ_FAIL) gb_set_error(e, "OSKAR payload: short read");
  else if (e) gb_set_error(e, "OSKAR payload staging failed (pinned memory or CUDA)");
  return e;
}

struct DevJob {
  int64_t file_off, n, dev_off;
  uint32_t crc, crc_hdr;
  int seq;  // position in the reference's read order
};

struct Ingest {
  std::vector<BlockDesc> blocks;
  std::vector<double> invl;
  std::vector<DevJob> jobs;
  int64_t raw_bytes = 0;
  int first_err = 0, first_err_seq = INT_MAX;
};

int64_t align256(int64_t x) { return (x + 255) & ~int64_t(255); }

// Timings of the calling thread's last read: host staging (pread + copies)
// wall ms, CRC kernel ms, reshuffle kernel ms (CUDA events on the read's
// stream), whole call wall ms.
thread_local double t_last[4] = {0, 0, 0, 0};

double wall_ms() {
  return std::chrono::duration<double, std::milli>(
             std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Reads the header and every block's small tags in the reference's order,
// locating (not reading) the large payloads; stops at the first failing step.
void plan_ingest(const VisData* vd, Ingest* in) {
  const oskar_Binary* b = vd->h;
  const int nb = vd->num_baselines, nc = vd->num_channels, T = vd->num_times;
  auto stop = [&](int seq, int code) {
    in->first_err = code;
    in->first_err_seq = seq;
  };
  int ntpb = 0, mtpb = 0, st;
  if ((st = read_tag(b, 0, T_INT, G_HEADER, H_NUM_TAGS_PER_BLOCK, 0, 4, &ntpb)) ||
      (st = read_tag(b, 0, T_INT, G_HEADER, H_MAX_TIMES_PER_BLOCK, 0, 4, &mtpb))) {
    stop(-1, st);
    return;
  }
  if (mtpb <= 0 || nb < 0 || nc < 0 || T < 0) {
    gb_set_error(GB_OSKAR_FORMAT_BAD, "OSKAR header: bad block or array sizes");
    stop(-1, GB_OSKAR_FORMAT_BAD);
    return;
  }
  const int nblocks = (T + mtpb - 1) / mtpb;
  const int64_t ntb = (int64_t)mtpb * nb;
  int search = 0;
  for (int blk = 0; blk < nblocks; blk++) {
    const int seq0 = blk * 8;
    const int64_t s0 = (int64_t)blk * ntpb;
    if (s0 >= 0 && s0 < (int64_t)b->chunks.size()) search = (int)s0;
    int dim[6] = {0, 0, 0, 0, 0, 0};
    double fr[2], tr[2];
    if ((st = read_tag(b, search, T_INT, G_BLOCK, B_DIM_START_AND_SIZE, blk, 24, dim)))
      return stop(seq0, st);
    if ((st = read_tag(b, search, T_DOUBLE, G_BLOCK, B_FREQ_REF_INC_HZ, blk, 16, fr)))
      return stop(seq0 + 1, st);
    if ((st = read_tag(b, search, T_DOUBLE, G_BLOCK, B_TIME_REF_INC_MJD, blk, 16, tr)))
      return stop(seq0 + 2, st);
    BlockDesc bd{};
    bd.t0 = dim[0];
    bd.nt = dim[2];
    bd.il = (int32_t)in->invl.size();
    double f = fr[0];
    for (int c = 0; c < nc; c++, f += fr[1]) in->invl.push_back(f / SPEED_OF_LIGHT);
    const int types[4] = {T_DOUBLE | T_COMPLEX | T_MATRIX, T_DOUBLE, T_DOUBLE, T_DOUBLE};
    const int tags[4] = {B_CROSS_CORR, B_UU, B_VV, B_WW};
    const int64_t cap[4] = {ntb * nc * 64, ntb * 8, ntb * 8, ntb * 8};
    const int64_t need[4] = {(int64_t)bd.nt * nb * nc * 64, (int64_t)bd.nt * nb * 8,
                             (int64_t)bd.nt * nb * 8, (int64_t)bd.nt * nb * 8};
    int64_t* dst[4] = {&bd.amp, &bd.u, &bd.v, &bd.w};
    for (int k = 0; k < 4; k++) {
      const int i = query(b, search, types[k], G_BLOCK, tags[k], blk);
      if (i < 0) {
        gb_set_error(GB_OSKAR_TAG_NOT_FOUND, "OSKAR block %d: payload tag %d not found", blk,
                     tags[k]);
        return stop(seq0 + 3 + k, GB_OSKAR_TAG_NOT_FOUND);
      }
      const Chunk& c = b->chunks[i];
      if (c.size > cap[k]) {
        gb_set_error(GB_OSKAR_MEMORY_NOT_ALLOCATED, "OSKAR block %d: payload %d too large",
                     blk, tags[k]);
        return stop(seq0 + 3 + k, GB_OSKAR_MEMORY_NOT_ALLOCATED);
      }
      if (c.size < need[k]) {
        gb_set_error(GB_OSKAR_FORMAT_BAD, "OSKAR block %d: payload %d shorter than its times",
                     blk, tags[k]);
        return stop(seq0 + 3 + k, GB_OSKAR_FORMAT_BAD);
      }
      *dst[k] = in->raw_bytes;
      if (c.size > 0)
        in->jobs.push_back({c.off, c.size, in->raw_bytes, c.crc, c.crc_hdr, seq0 + 3 + k});
      in->raw_bytes = align256(in->raw_bytes + c.size);
    }
    if (bd.nt < 0 || bd.nt > mtpb || bd.t0 < 0 || (int64_t)bd.t0 + bd.nt > T || dim[1] != 0) {
      gb_set_error(GB_OSKAR_FORMAT_BAD, "OSKAR block %d: times/channels outside the header's",
                   blk);
      return stop(seq0 + 7, GB_OSKAR_FORMAT_BAD);
    }
    in->blocks.push_back(bd);
  }
}

int cuda_fail(cudaError_t e, const char* what) {
  gb_set_error(GB_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  return GB_ERR_CUDA;
}

#define OSK_CUDA(call, what)                 \
  do {                                       \
    cudaError_t e_ = (call);                 \
    if (e_ != cudaSuccess) {                 \
      rc = cuda_fail(e_, what);              \
      goto done;                             \
    }                                        \
  } while (0)

int check_vd(const VisData* vd) {
  if (!vd || !vd->h) {
    gb_set_error(GB_ERR_ARG, "VisData without an open file");
    return GB_ERR_ARG;
  }
  return 0;
}

// The extraction entries need only the counts, not the open file.
int check_counts(const VisData* vd) {
  if (!vd || vd->num_times < 0 || vd->num_channels < 0 || vd->num_times_baselines < 0) {
    gb_set_error(GB_ERR_ARG, "VisData missing or with negative counts");
    return GB_ERR_ARG;
  }
  return 0;
}

// Reads every block to the device; d_amps / d_uvws receive the reshuffled
// arrays, gm_host (6) and blw_host (2 * num_baselines) the extrema keys.
int ingest(const VisData* vd, double* d_amps, double* d_uvws, Metrix* mp, WMaxMin* bl_ws,
           cudaStream_t s) {
  int rc = check_vd(vd);
  if (rc) return rc;
  const double t_start = wall_ms();
  const int nb = vd->num_baselines, nc = vd->num_channels, T = vd->num_times;
  cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
  double t_stage = 0;
  Ingest in;
  plan_ingest(vd, &in);
  if (in.first_err_seq == -1) return in.first_err;
  // keep the payloads before the first failing step (their CRC may fail earlier)
  std::vector<DevJob> jobs;
  for (const DevJob& j : in.jobs)
    if (j.seq < in.first_err_seq) jobs.push_back(j);
  const int tiles = (nb + kRB - 1) / kRB;
  const int64_t items = (int64_t)in.blocks.size() * nc * tiles;
  int per_sm = 0;  // persistent: as many CTAs as fit at once
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_oskar_reshuffle, 256, 0) !=
          cudaSuccess || per_sm < 1)
    per_sm = 1;
  const int n_cta = (int)std::min<int64_t>(items, (int64_t)gb::sm_count() * per_sm);
  const int64_t gm_off = align256(in.raw_bytes);
  const int64_t blw_off = align256(gm_off + (int64_t)n_cta * 48);
  const int64_t crc_off = align256(blw_off + (int64_t)std::max(nb, 0) * 16);
  const int64_t job_off = align256(crc_off + (int64_t)jobs.size() * 4);
  const int64_t pw_off = align256(job_off + (int64_t)jobs.size() * sizeof(CrcJob));
  const int64_t blk_off = align256(pw_off + (kCrcPowers + 3) * 32 * 4);
  const int64_t il_off = align256(blk_off + (int64_t)in.blocks.size() * sizeof(BlockDesc));
  const int64_t total = align256(il_off + (int64_t)in.invl.size() * 8);
  uint8_t* d = nullptr;
  std::vector<unsigned long long> part(6 * (size_t)n_cta), keys(2 * (size_t)std::max(nb, 0));
  std::vector<uint32_t> crc_out(jobs.size());
  std::vector<CrcJob> cj(jobs.size());
  const std::vector<uint32_t> pw = crc_device_maps();
  std::vector<Piece> pieces;
  int64_t chunks = 0;
  int crc_fail_seq = INT_MAX;
  for (size_t j = 0; j < jobs.size(); j++) {
    const DevJob& J = jobs[j];
    cj[j].off = J.dev_off;
    cj[j].n = J.n;
    cj[j].first_chunk = chunks;
    const int64_t k = (J.n + kCrcChunk - 1) >> kCrcChunkLog;
    const Op last = zeros_op((uint64_t)(J.n - (k - 1) * kCrcChunk));
    memcpy(cj[j].last, last.c, 128);
    chunks += k;
    for (int64_t o = 0; o < J.n; o += kSlot)
      pieces.push_back({J.file_off + o, J.dev_off + o, std::min(kSlot, J.n - o)});
  }
  OSK_CUDA(cudaMallocAsync((void**)&d, (size_t)total, s), "cudaMallocAsync(OSKAR staging)");
  OSK_CUDA(cudaMemsetAsync(d + crc_off, 0, jobs.size() * 4 + 4, s), "memset");
  if (!jobs.empty())
    OSK_CUDA(cudaMemcpyAsync(d + job_off, cj.data(), cj.size() * sizeof(CrcJob),
                             cudaMemcpyHostToDevice, s), "jobs H2D");
  OSK_CUDA(cudaMemcpyAsync(d + pw_off, pw.data(), pw.size() * 4, cudaMemcpyHostToDevice, s),
           "powers H2D");
  if (!in.blocks.empty())
    OSK_CUDA(cudaMemcpyAsync(d + blk_off, in.blocks.data(), in.blocks.size() * sizeof(BlockDesc),
                             cudaMemcpyHostToDevice, s), "blocks H2D");
  if (!in.invl.empty())
    OSK_CUDA(cudaMemcpyAsync(d + il_off, in.invl.data(), in.invl.size() * 8,
                             cudaMemcpyHostToDevice, s), "1/lambda H2D");
  for (int k = 0; k < 3; k++) OSK_CUDA(cudaEventCreate(&ev[k]), "cudaEventCreate");
  // the reader threads copy on their own streams: the allocation must exist first
  OSK_CUDA(cudaStreamSynchronize(s), "stream sync");
  t_stage = wall_ms();
  rc = stream_pieces(vd->h->fd, pieces, d);
  t_stage = wall_ms() - t_stage;
  if (rc) goto done;
  OSK_CUDA(cudaEventRecord(ev[0], s), "cudaEventRecord");
  {
    const unsigned long long kmax = host_key(-1e12), kmin = host_key(1e12);
    if (nb > 0) {
      k_oskar_init_extrema<<<(unsigned)((nb + 255) / 256), 256, 0, s>>>(
          (unsigned long long*)(d + blw_off), nb, kmax, kmin);
      OSK_CUDA(cudaGetLastError(), "k_oskar_init_extrema");
    }
  }
  if (chunks > 0) {
    const int64_t grid =
        std::min<int64_t>((4 * chunks + 255) / 256, (int64_t)gb::sm_count() * 64);
    k_crc32c<<<(unsigned)grid, 256, 0, s>>>(d, (const CrcJob*)(d + job_off), (int)jobs.size(),
                                            chunks, (const uint32_t*)(d + pw_off),
                                            (uint32_t*)(d + crc_off));
    OSK_CUDA(cudaGetLastError(), "k_crc32c");
  }
  OSK_CUDA(cudaEventRecord(ev[1], s), "cudaEventRecord");
  if (n_cta > 0) {
    k_oskar_reshuffle<<<(unsigned)n_cta, 256, 0, s>>>(
        d, (const BlockDesc*)(d + blk_off), (int32_t)in.blocks.size(),
        (const double*)(d + il_off), nb, nc, T, d_amps, d_uvws,
        (unsigned long long*)(d + gm_off), (unsigned long long*)(d + blw_off));
    OSK_CUDA(cudaGetLastError(), "k_oskar_reshuffle");
  }
  OSK_CUDA(cudaEventRecord(ev[2], s), "cudaEventRecord");
  if (n_cta > 0)
    OSK_CUDA(cudaMemcpyAsync(part.data(), d + gm_off, part.size() * 8, cudaMemcpyDeviceToHost,
                             s), "D2H");
  if (nb > 0)
    OSK_CUDA(cudaMemcpyAsync(keys.data(), d + blw_off, (size_t)nb * 16,
                             cudaMemcpyDeviceToHost, s), "D2H");
  if (!jobs.empty())
    OSK_CUDA(cudaMemcpyAsync(crc_out.data(), d + crc_off, jobs.size() * 4,
                             cudaMemcpyDeviceToHost, s), "D2H");
  OSK_CUDA(cudaStreamSynchronize(s), "stream sync");
  {
    float a = 0, b = 0;
    cudaEventElapsedTime(&a, ev[0], ev[1]);
    cudaEventElapsedTime(&b, ev[1], ev[2]);
    t_last[0] = t_stage;
    t_last[1] = a;
    t_last[2] = b;
  }
  for (size_t j = 0; j < jobs.size(); j++) {
    const DevJob& J = jobs[j];
    if (!J.crc) continue;
    const uint32_t code = zeros_apply((uint64_t)J.n, reopen(J.crc_hdr)) ^ crc_out[j] ^ kInit;
    if (code != J.crc && J.seq < crc_fail_seq) crc_fail_seq = J.seq;
  }
  if (crc_fail_seq < in.first_err_seq) {
    gb_set_error(GB_OSKAR_CRC_FAIL, "OSKAR payload: CRC mismatch (block %d)", crc_fail_seq / 8);
    rc = GB_OSKAR_CRC_FAIL;
  } else {
    rc = in.first_err;
  }
  if (mp) {
    // the reference's start values -1e12 / 1e12 take part like any value
    unsigned long long g[6] = {host_key(-1e12), host_key(-1e12), host_key(-1e12),
                               host_key(1e12), host_key(1e12), host_key(1e12)};
    for (int c = 0; c < n_cta; c++)
      for (int k = 0; k < 6; k++)
        g[k] = k < 3 ? std::max(g[k], part[6 * c + k]) : std::min(g[k], part[6 * c + k]);
    mp->maxu = key_value(g[0]);
    mp->maxv = key_value(g[1]);
    mp->maxw = key_value(g[2]);
    mp->minu = key_value(g[3]);
    mp->minv = key_value(g[4]);
    mp->minw = key_value(g[5]);
  }
  if (bl_ws)
    for (int i = 0; i < nb; i++) {
      bl_ws[i].maxw = key_value(keys[2 * i]);
      bl_ws[i].minw = key_value(keys[2 * i + 1]);
    }
done:
  if (d) {
    cudaFreeAsync(d, s);
    cudaStreamSynchronize(s);
  }
  for (int k = 0; k < 3; k++)
    if (ev[k]) cudaEventDestroy(ev[k]);
  t_last[3] = wall_ms() - t_start;
  return rc;
}

}  // namespace

extern "C" int gb_oskar_last_timings(double* out4) {
  if (!out4) {
    gb_set_error(GB_ERR_ARG, "gb_oskar_last_timings: NULL output");
    return GB_ERR_ARG;
  }
  for (int k = 0; k < 4; k++) out4[k] = t_last[k];
  return 0;
}

// ================================================================ C ABI
extern "C" void* _aligned_malloc(size_t size, size_t alignment) {
  void* p = nullptr;
  const int e = posix_memalign(&p, alignment, size);
  errno = e;
  return e ? nullptr : p;
}

extern "C" int mkFromFile(VisData* vdp, const char* filename) {
  if (!vdp || !filename) {
    gb_set_error(GB_ERR_ARG, "mkFromFile: NULL argument");
    return GB_ERR_ARG;
  }
  oskar_Binary* b = nullptr;
  int st = bin_open(filename, &b);
  if (st) return st;
  int amp_type = 0, nt = 0, nc = 0, ns = 0;
  double fr[2] = {0, 0}, tm[2] = {0, 0}, bw = 0, avg = 0, pc[2] = {0, 0}, tc[3] = {0, 0, 0};
  if ((st = read_tag(b, 0, T_INT, G_HEADER, H_AMP_TYPE, 0, 4, &amp_type)) ||
      (st = read_tag(b, 0, T_INT, G_HEADER, H_NUM_TIMES_TOTAL, 0, 4, &nt)) ||
      (st = read_tag(b, 0, T_INT, G_HEADER, H_NUM_CHANNELS, 0, 4, &nc)) ||
      (st = read_tag(b, 0, T_INT, G_HEADER, H_NUM_STATIONS, 0, 4, &ns))) {
    delete b;
    return st;
  }
  if ((amp_type & 0x0F) != T_DOUBLE) {
    delete b;
    gb_set_error(GB_OSKAR_NOT_DOUBLE, "%s: amplitudes are not double precision", filename);
    return GB_OSKAR_NOT_DOUBLE;
  }
  if ((st = read_tag(b, 0, T_DOUBLE, G_HEADER, H_FREQ_START_HZ, 0, 8, &fr[0])) ||
      (st = read_tag(b, 0, T_DOUBLE, G_HEADER, H_FREQ_INC_HZ, 0, 8, &fr[1])) ||
      (st = read_tag(b, 0, T_DOUBLE, G_HEADER, H_CHANNEL_BW_HZ, 0, 8, &bw)) ||
      (st = read_tag(b, 0, T_DOUBLE, G_HEADER, H_TIME_START_MJD, 0, 8, &tm[0])) ||
      (st = read_tag(b, 0, T_DOUBLE, G_HEADER, H_TIME_INC_SEC, 0, 8, &tm[1])) ||
      (st = read_tag(b, 0, T_DOUBLE, G_HEADER, H_TIME_AVERAGE_SEC, 0, 8, &avg)) ||
      (st = read_tag(b, 0, T_DOUBLE, G_HEADER, H_PHASE_CENTRE, 0, 16, pc)) ||
      (st = read_tag(b, 0, T_DOUBLE, G_HEADER, H_TELESCOPE_CENTRE, 0, 24, tc))) {
    delete b;
    return st;
  }
  const int64_t nbl = (int64_t)ns * (ns - 1) / 2, ntb = nbl * nt, np = ntb * nc;
  if (ns < 0 || nt < 0 || nc < 0 || np > INT_MAX || ntb > INT_MAX) {
    delete b;
    gb_set_error(GB_ERR_CAPACITY, "%s: point count does not fit the reader's int fields",
                 filename);
    return GB_ERR_CAPACITY;
  }
  vdp->h = b;
  vdp->num_baselines = (int)nbl;
  vdp->num_channels = nc;
  vdp->num_stations = ns;
  vdp->num_times = nt;
  vdp->num_times_baselines = (int)ntb;
  vdp->num_points = (int)np;
  vdp->phase_centre[0] = pc[0];
  vdp->phase_centre[1] = pc[1];
  for (int i = 0; i < 3; i++) vdp->telescope_centre[i] = tc[i];
  vdp->freq_start_inc[0] = fr[0];
  vdp->freq_start_inc[1] = fr[1];
  vdp->time_start_inc[0] = tm[0];
  vdp->time_start_inc[1] = tm[1];
  vdp->channel_bandwidth_hz = bw;
  vdp->time_average_sec = avg;
  return 0;
}

extern "C" void freeBinHandler(VisData* vdp) {
  if (!vdp) return;
  delete vdp->h;
  vdp->h = nullptr;
}

extern "C" int gb_oskar_read_device(const VisData* vdp, double* d_amps, double* d_uvws,
                                    Metrix* mp, WMaxMin* bl_ws, void* stream) {
  int rc = check_vd(vdp);
  if (rc) return rc;
  if (vdp->num_points > 0 && (!d_amps || !d_uvws)) {
    gb_set_error(GB_ERR_ARG, "gb_oskar_read_device: NULL output");
    return GB_ERR_ARG;
  }
  return ingest(vdp, d_amps, d_uvws, mp, bl_ws, (cudaStream_t)stream);
}

extern "C" int readAndReshuffle(const VisData* vdp, double* amps, double* uvws, Metrix* mp,
                                WMaxMin* bl_ws) {
  int rc = check_vd(vdp);
  if (rc) return rc;
  const int64_t np = vdp->num_points;
  if (np > 0 && (!amps || !uvws)) {
    gb_set_error(GB_ERR_ARG, "readAndReshuffle: NULL output");
    return GB_ERR_ARG;
  }
  cudaStream_t s;
  if ((rc = gb::stage_stream(&s))) return rc;
  double* d = nullptr;
  const size_t bytes = (size_t)np * 88;
  if (np > 0) {
    const cudaError_t e = cudaMallocAsync((void**)&d, bytes, s);
    if (e != cudaSuccess) {
      gb_set_error(GB_ERR_NOMEM, "readAndReshuffle: device outputs: %s", cudaGetErrorString(e));
      return GB_ERR_NOMEM;
    }
  }
  rc = ingest(vdp, d, d ? d + 8 * np : nullptr, mp, bl_ws, s);
  if (np > 0) {
    if (rc == 0) {
      cudaError_t e = cudaMemcpyAsync(amps, d, (size_t)np * 64, cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(uvws, d + 8 * np, (size_t)np * 24, cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
      if (e != cudaSuccess) rc = cuda_fail(e, "readAndReshuffle: D2H");
    }
    cudaFreeAsync(d, s);
    cudaStreamSynchronize(s);
  }
  return rc;
}

extern "C" int gb_oskar_records(const VisData* vdp, const double* d_amps, const double* d_uvws,
                                int32_t freq, int32_t pol, int64_t dom_low, int64_t dom_high,
                                int32_t flags, double* d_records, void* stream) {
  int rc = check_counts(vdp);
  if (rc) return rc;
  const int64_t T = vdp->num_times, total = (int64_t)vdp->num_times_baselines;
  if (freq < 0 || freq >= vdp->num_channels || pol < 0 || pol > 3 || dom_low < 0 ||
      dom_high > total || dom_high < dom_low || (T > 0 && dom_low % T != 0)) {
    gb_set_error(GB_ERR_ARG,
                 "gb_oskar_records: channel/polarisation out of range or region not "
                 "baseline-aligned inside [0, %lld)", (long long)total);
    return GB_ERR_ARG;
  }
  const int64_t n = dom_high - dom_low;
  if (n == 0) return 0;
  if (!d_amps || !d_uvws || !d_records) {
    gb_set_error(GB_ERR_ARG, "gb_oskar_records: NULL pointer");
    return GB_ERR_ARG;
  }
  const unsigned g = (unsigned)std::min<int64_t>((n + 255) / 256, (int64_t)gb::sm_count() * 32);
  k_oskar_records<<<g, 256, 0, (cudaStream_t)stream>>>(d_amps, d_uvws, (int32_t)T,
                                                       vdp->num_channels, freq, pol, dom_low, n,
                                                       flags & GB_OSKAR_REFERENCE_UVW_INDEX,
                                                       d_records);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? 0 : cuda_fail(e, "k_oskar_records");
}

extern "C" int gb_oskar_extract(const VisData* vdp, const double* d_amps, const double* d_uvws,
                                int32_t freq, int32_t pol, double* d_uvw, void* d_vis,
                                int32_t vis_f64, void* stream) {
  int rc = check_counts(vdp);
  if (rc) return rc;
  if (freq < 0 || freq >= vdp->num_channels || pol < 0 || pol > 3) {
    gb_set_error(GB_ERR_ARG, "gb_oskar_extract: channel or polarisation out of range");
    return GB_ERR_ARG;
  }
  const int64_t n = vdp->num_times_baselines;
  if (n == 0) return 0;
  if (!d_amps || !d_uvws || !d_uvw || !d_vis) {
    gb_set_error(GB_ERR_ARG, "gb_oskar_extract: NULL pointer");
    return GB_ERR_ARG;
  }
  const unsigned g = (unsigned)std::min<int64_t>((n + 255) / 256, (int64_t)gb::sm_count() * 32);
  if (vis_f64)
    k_oskar_extract<double2><<<g, 256, 0, (cudaStream_t)stream>>>(
        d_amps, d_uvws, vdp->num_channels, freq, pol, n, d_uvw, (double2*)d_vis);
  else
    k_oskar_extract<float2><<<g, 256, 0, (cudaStream_t)stream>>>(
        d_amps, d_uvws, vdp->num_channels, freq, pol, n, d_uvw, (float2*)d_vis);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? 0 : cuda_fail(e, "k_oskar_extract");
}

extern "C" int gb_crc32c_device(const void* d_data, int64_t n, uint32_t code, uint32_t* out,
                                void* stream) {
  if (!out || n < 0 || (n > 0 && (!d_data || ((uintptr_t)d_data & 15)))) {
    gb_set_error(GB_ERR_ARG, "gb_crc32c_device: NULL output, negative size or data not "
                             "16-byte aligned");
    return GB_ERR_ARG;
  }
  if (n == 0) {
    *out = code;  // no bytes: the code is returned as given
    return 0;
  }
  if (((n + kCrcChunk - 1) >> kCrcChunkLog) >= (int64_t(1) << kCrcPowers)) {
    gb_set_error(GB_ERR_CAPACITY, "gb_crc32c_device: more than 2^40 bytes");
    return GB_ERR_CAPACITY;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const int64_t k = (n + kCrcChunk - 1) >> kCrcChunkLog;
  CrcJob job;
  job.off = 0;
  job.n = n;
  job.first_chunk = 0;
  memcpy(job.last, zeros_op((uint64_t)(n - (k - 1) * kCrcChunk)).c, 128);
  const std::vector<uint32_t> pw = crc_device_maps();
  uint8_t* d = nullptr;
  uint32_t r = 0;
  int rc = 0;
  OSK_CUDA(cudaMallocAsync((void**)&d, 256 + sizeof(CrcJob) + pw.size() * 4, s),
           "cudaMallocAsync");
  OSK_CUDA(cudaMemsetAsync(d, 0, 4, s), "memset");
  OSK_CUDA(cudaMemcpyAsync(d + 256, &job, sizeof(job), cudaMemcpyHostToDevice, s), "H2D");
  OSK_CUDA(cudaMemcpyAsync(d + 256 + sizeof(CrcJob), pw.data(), pw.size() * 4,
                           cudaMemcpyHostToDevice, s), "H2D");
  {
    const int64_t grid = std::min<int64_t>((4 * k + 255) / 256, (int64_t)gb::sm_count() * 64);
    k_crc32c<<<(unsigned)grid, 256, 0, s>>>((const uint8_t*)d_data, (const CrcJob*)(d + 256), 1,
                                            k, (const uint32_t*)(d + 256 + sizeof(CrcJob)),
                                            (uint32_t*)d);
    OSK_CUDA(cudaGetLastError(), "k_crc32c");
  }
  OSK_CUDA(cudaMemcpyAsync(&r, d, 4, cudaMemcpyDeviceToHost, s), "D2H");
  OSK_CUDA(cudaStreamSynchronize(s), "stream sync");
  *out = zeros_apply((uint64_t)n, reopen(code)) ^ r ^ kInit;
done:
  if (d) {
    cudaFreeAsync(d, s);
    cudaStreamSynchronize(s);
  }
  return rc;
}
