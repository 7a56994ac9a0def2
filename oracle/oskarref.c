/* OSKAR 2.6 visibility files: the oracle's C restatement of the reference
 * reader, plus a writer of that layout.  TEST INFRASTRUCTURE ONLY: tests,
 * the smoke check and the CPU-baseline leg of bench.py use it as the checker;
 * nothing in rc_gb300 links or calls it.
 *
 * Restated from SKA-ScienceDataProcessor/RC (own code, same rules):
 *   - the container (MS6/kernel/oskar/oskar_binary/private_binary.h:44-183):
 *     a 64-byte file header ("OSKARBIN\0", format version), then chunks of a
 *     20-byte tag ('T', 0x40 + version, 'G', element size, flags, type code,
 *     group id, tag id, int32 user index, int64 block size), optional group
 *     and tag names (extended tags, flag bit 7), the payload, and a 4-byte
 *     CRC-32C when flag bit 6 is set; flag bits 0-4 must be zero;
 *   - the index scan, its checks and status codes
 *     (oskar_binary/src/oskar_binary_create.c:48-282, oskar_binary.h:96-114);
 *   - tag lookup from the search start (oskar_binary_query.c:38-68, 123-131)
 *     and payload reads with the CRC check (oskar_binary_read.c:38-101);
 *   - CRC-32C (oskar_crc.c:45-160): reflected polynomial 0x82F63B78, initial
 *     value and final xor 0xFFFFFFFF, and the update rule that re-opens a
 *     finished code with the final xor unless the code equals the initial
 *     value.  Computed here by the published slicing-by-8 table method;
 *   - mkFromFile and readAndReshuffle (MS6/kernel/oskar/OskarBinReader.cpp:
 *     149-238 and 246-413): header fields, the double-precision amplitude
 *     check (0xdeadbeef), per-block wavelength scaling 1/lambda_c =
 *     f_c / c with f_c accumulated by repeated addition of the increment, the
 *     [t][c][b] -> [b][t][c] reshuffle of 4-polarisation amplitudes and of
 *     u,v,w (metres x 1/lambda), the global u/v/w extrema (initial -1e12 /
 *     1e12, NaN never replaces a value) and per-baseline w extrema.
 * The writer emits the tags OskarBinReader.cpp:67-100 names, in header group
 * 11 and block group 12, as the same container.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define ORC_C_LIGHT 299792458.0

enum {
  ST_OPEN_FAIL = -100, ST_SEEK_FAIL = -101, ST_READ_FAIL = -102, ST_WRITE_FAIL = -103,
  ST_FILE_INVALID = -106, ST_FORMAT_BAD = -107, ST_ENDIAN = -108, ST_VERSION = -109,
  ST_TYPE = -110, ST_INT = -111, ST_FLOAT = -112, ST_DOUBLE = -113, ST_MEMORY = -114,
  ST_NOT_FOUND = -115, ST_CRC = -118
};
enum { T_CHAR = 0x01, T_INT = 0x02, T_SINGLE = 0x04, T_DOUBLE = 0x08, T_COMPLEX = 0x20,
       T_MATRIX = 0x40 };
enum { G_HEADER = 11, G_BLOCK = 12 };
enum { H_TELESCOPE_PATH = 1, H_NUM_TAGS_PER_BLOCK, H_WRITE_AUTOCORR, H_AMP_TYPE,
       H_MAX_TIMES_PER_BLOCK, H_NUM_TIMES_TOTAL, H_NUM_CHANNELS, H_NUM_STATIONS,
       H_FREQ_START_HZ, H_FREQ_INC_HZ, H_CHANNEL_BW_HZ, H_TIME_START_MJD, H_TIME_INC_SEC,
       H_TIME_AVERAGE_SEC, H_PHASE_CENTRE, H_TELESCOPE_CENTRE, H_STATION_X, H_STATION_Y,
       H_STATION_Z };
enum { B_DIM_START_AND_SIZE = 1, B_FREQ_REF_INC_HZ, B_TIME_REF_INC_MJD, B_AUTO_CORR,
       B_CROSS_CORR, B_UU, B_VV, B_WW };

/* ------------------------------------------------------------------ CRC-32C */
static uint32_t g_tab[8][256];
static int g_tab_ready = 0;

static void crc_tables(void) {
  if (g_tab_ready) return;
  for (uint32_t i = 0; i < 256; i++) {
    uint32_t c = i;
    for (int k = 0; k < 8; k++) c = (c >> 1) ^ (0x82F63B78u & (0u - (c & 1u)));
    g_tab[0][i] = c;
  }
  for (int k = 1; k < 8; k++)
    for (int i = 0; i < 256; i++)
      g_tab[k][i] = (g_tab[k - 1][i] >> 8) ^ g_tab[0][g_tab[k - 1][i] & 0xFF];
  g_tab_ready = 1;
}

/* register update over n bytes (no initial or final xor) */
static uint32_t crc_raw(uint32_t s, const uint8_t* p, size_t n) {
  while (n >= 8) {
    const uint32_t lo = s ^ ((uint32_t)p[0] | (uint32_t)p[1] << 8 | (uint32_t)p[2] << 16 |
                             (uint32_t)p[3] << 24);
    const uint32_t hi = (uint32_t)p[4] | (uint32_t)p[5] << 8 | (uint32_t)p[6] << 16 |
                        (uint32_t)p[7] << 24;
    s = g_tab[7][lo & 0xFF] ^ g_tab[6][(lo >> 8) & 0xFF] ^ g_tab[5][(lo >> 16) & 0xFF] ^
        g_tab[4][lo >> 24] ^ g_tab[3][hi & 0xFF] ^ g_tab[2][(hi >> 8) & 0xFF] ^
        g_tab[1][(hi >> 16) & 0xFF] ^ g_tab[0][hi >> 24];
    p += 8;
    n -= 8;
  }
  while (n--) s = (s >> 8) ^ g_tab[0][(s ^ *p++) & 0xFF];
  return s;
}

/* the container's update of a finished code */
static uint32_t crc_update(uint32_t code, const void* p, size_t n) {
  crc_tables();
  const uint32_t s = code == 0xFFFFFFFFu ? code : code ^ 0xFFFFFFFFu;
  return crc_raw(s, (const uint8_t*)p, n) ^ 0xFFFFFFFFu;
}

uint32_t orc_crc32c(const void* p, size_t n) { return crc_update(0xFFFFFFFFu, p, n); }
uint32_t orc_crc32c_update(uint32_t code, const void* p, size_t n) {
  return crc_update(code, p, n);
}

/* ------------------------------------------------------------------ reader */
typedef struct {
  int ext, type, group, tag, user;
  long long off, size;
  uint32_t crc, crc_hdr;
  char gname[256], tname[256];
} Chunk;

typedef struct {
  FILE* f;
  int n, cap, search;
  Chunk* c;
} Bin;

static void bin_free(Bin* b) {
  if (!b) return;
  if (b->f) fclose(b->f);
  free(b->c);
  free(b);
}

static int32_t le32(const uint8_t* p) {
  return (int32_t)((uint32_t)p[0] | (uint32_t)p[1] << 8 | (uint32_t)p[2] << 16 |
                   (uint32_t)p[3] << 24);
}
static int64_t le64(const uint8_t* p) {
  uint64_t v = 0;
  for (int i = 7; i >= 0; i--) v = v << 8 | p[i];
  return (int64_t)v;
}

static Bin* bin_open(const char* path, int* status) {
  uint8_t hdr[64];
  FILE* f = fopen(path, "rb");
  if (!f) {
    *status = ST_OPEN_FAIL;
    return NULL;
  }
  if (fread(hdr, 64, 1, f) != 1) {
    fclose(f);
    *status = ST_READ_FAIL;
    return NULL;
  }
  if (memcmp(hdr, "OSKARBIN", 8) != 0) {
    fclose(f);
    *status = ST_FILE_INVALID;
    return NULL;
  }
  const int version = (signed char)hdr[9];
  if (version > 2) {
    fclose(f);
    *status = ST_VERSION;
    return NULL;
  }
  if (version == 1) {
    /* little-endian host; the last failing size check decides the code */
    if (hdr[10] != 0) {
      fclose(f);
      *status = ST_ENDIAN;
      return NULL;
    }
    if (hdr[12] != 4) *status = ST_INT;
    if (hdr[14] != 4) *status = ST_FLOAT;
    if (hdr[15] != 8) *status = ST_DOUBLE;
    if (*status) {
      fclose(f);
      return NULL;
    }
  }
  Bin* b = (Bin*)calloc(1, sizeof(Bin));
  b->f = f;
  for (int i = 0;; i++) {
    uint8_t t[20];
    if (fread(t, 20, 1, f) != 1) break;
    if (t[0] != 'T' || t[2] != 'G' || (t[4] & 0x1F) != 0) {
      *status = ST_FILE_INVALID;
      break;
    }
    const int fv = (int)(signed char)t[1] - 0x40;
    if (fv < 1 || fv > 2) {
      *status = ST_VERSION;
      break;
    }
    if (fv > 1) {
      int es = (signed char)t[3];
      const int ty = t[5];
      if (ty & T_MATRIX) es /= 4;
      if (ty & T_COMPLEX) es /= 2;
      /* a failed size check marks the file bad but the scan goes on */
      if (ty & T_CHAR) {
        if (es != 1) *status = ST_FORMAT_BAD;
      } else if (ty & T_INT) {
        if (es != 4) *status = ST_INT;
      } else if (ty & T_SINGLE) {
        if (es != 4) *status = ST_FLOAT;
      } else if (ty & T_DOUBLE) {
        if (es != 8) *status = ST_DOUBLE;
      } else {
        *status = ST_TYPE;
      }
    }
    if (b->n == b->cap) {
      b->cap = b->cap ? 2 * b->cap : 64;
      b->c = (Chunk*)realloc(b->c, (size_t)b->cap * sizeof(Chunk));
    }
    Chunk* c = &b->c[i];
    memset(c, 0, sizeof(*c));
    uint32_t crc = orc_crc32c(t, 20);
    c->type = t[5];
    c->group = t[6];
    c->tag = t[7];
    c->user = le32(t + 8);
    const long long block = (long long)le64(t + 12);
    c->size = block - ((t[4] & 0x40) ? 4 : 0);
    if (t[4] & 0x80) {
      c->ext = 1;
      c->size -= (long long)t[6] + t[7];
    }
    if (c->size < 0) {
      /* a block too short for its own names and code (the reference would
         seek backwards here) */
      *status = ST_FILE_INVALID;
      break;
    }
    if (c->ext) {
      if (fread(c->gname, t[6], 1, f) != 1 || fread(c->tname, t[7], 1, f) != 1) {
        *status = ST_FILE_INVALID;
        break;
      }
      crc = crc_update(crc, c->gname, t[6]);
      crc = crc_update(crc, c->tname, t[7]);
    }
    c->off = ftell(f);
    if (fseek(f, (long)c->size, SEEK_CUR) != 0) {
      *status = ST_FILE_INVALID;
      break;
    }
    c->crc_hdr = crc;
    if (t[4] & 0x40) {
      uint8_t cb[4];
      if (fread(cb, 4, 1, f) != 1) {
        *status = ST_FILE_INVALID;
        break;
      }
      c->crc = (uint32_t)le32(cb);
    }
    b->n = i + 1;
  }
  if (*status) {
    bin_free(b);
    return NULL;
  }
  return b;
}

static int bin_read_n(Bin* b, int type, int group, int tag, int user, size_t cap, void* dst,
                      size_t* got) {
  int i;
  *got = 0;
  for (i = b->search; i < b->n; i++) {
    const Chunk* c = &b->c[i];
    if (!c->ext && c->type == type && c->group == group && c->tag == tag && c->user == user)
      break;
  }
  if (i >= b->n) return ST_NOT_FOUND;
  const Chunk* c = &b->c[i];
  if (c->size == 0) return 0;
  if (!dst || cap < (size_t)c->size) return ST_MEMORY;
  if (fseek(b->f, (long)c->off, SEEK_SET) != 0) return ST_SEEK_FAIL;
  if (fread(dst, 1, (size_t)c->size, b->f) != (size_t)c->size) return ST_READ_FAIL;
  if (c->crc && crc_update(c->crc_hdr, dst, (size_t)c->size) != c->crc) return ST_CRC;
  *got = (size_t)c->size;
  return 0;
}

static int bin_read(Bin* b, int type, int group, int tag, int user, size_t cap, void* dst) {
  size_t got;
  return bin_read_n(b, type, group, tag, user, cap, dst, &got);
}

/* Fields of the reference's VisData after the handle, in its order. */
typedef struct {
  int num_baselines, num_channels, num_stations, num_times, num_times_baselines, num_points;
  double phase_centre[2], telescope_centre[3], freq_start_inc[2], time_start_inc[2],
      channel_bandwidth_hz, time_average_sec;
} orc_vis_header;

static int read_header(Bin* b, orc_vis_header* h) {
  int amp_type = 0, st;
  memset(h, 0, sizeof(*h));
  if ((st = bin_read(b, T_INT, G_HEADER, H_AMP_TYPE, 0, 4, &amp_type))) return st;
  if ((st = bin_read(b, T_INT, G_HEADER, H_NUM_TIMES_TOTAL, 0, 4, &h->num_times))) return st;
  if ((st = bin_read(b, T_INT, G_HEADER, H_NUM_CHANNELS, 0, 4, &h->num_channels))) return st;
  if ((st = bin_read(b, T_INT, G_HEADER, H_NUM_STATIONS, 0, 4, &h->num_stations))) return st;
  if ((amp_type & 0x0F) != T_DOUBLE) return (int)0xdeadbeefu;
  if ((st = bin_read(b, T_DOUBLE, G_HEADER, H_FREQ_START_HZ, 0, 8, &h->freq_start_inc[0])))
    return st;
  if ((st = bin_read(b, T_DOUBLE, G_HEADER, H_FREQ_INC_HZ, 0, 8, &h->freq_start_inc[1])))
    return st;
  if ((st = bin_read(b, T_DOUBLE, G_HEADER, H_CHANNEL_BW_HZ, 0, 8, &h->channel_bandwidth_hz)))
    return st;
  if ((st = bin_read(b, T_DOUBLE, G_HEADER, H_TIME_START_MJD, 0, 8, &h->time_start_inc[0])))
    return st;
  if ((st = bin_read(b, T_DOUBLE, G_HEADER, H_TIME_INC_SEC, 0, 8, &h->time_start_inc[1])))
    return st;
  if ((st = bin_read(b, T_DOUBLE, G_HEADER, H_TIME_AVERAGE_SEC, 0, 8, &h->time_average_sec)))
    return st;
  if ((st = bin_read(b, T_DOUBLE, G_HEADER, H_PHASE_CENTRE, 0, 16, h->phase_centre))) return st;
  if ((st = bin_read(b, T_DOUBLE, G_HEADER, H_TELESCOPE_CENTRE, 0, 24, h->telescope_centre)))
    return st;
  h->num_baselines = h->num_stations * (h->num_stations - 1) / 2;
  h->num_times_baselines = h->num_times * h->num_baselines;
  h->num_points = h->num_times_baselines * h->num_channels;
  return 0;
}

int orc_oskar_header(const char* path, orc_vis_header* h) {
  int st = 0;
  Bin* b = bin_open(path, &st);
  if (!b) return st;
  st = read_header(b, h);
  bin_free(b);
  return st;
}

static double dmax(double a, double b) { return a < b ? b : a; }
static double dmin(double a, double b) { return b < a ? b : a; }

/* mkFromFile + readAndReshuffle.  amps: num_points x 8 doubles, uvws:
 * num_points x 3, metrix: maxu maxv maxw minu minv minw, blws: num_baselines x
 * (maxw, minw).  Returns the reference's status. */
int orc_oskar_read(const char* path, double* amps, double* uvws, double* metrix, double* blws) {
  int st = 0;
  orc_vis_header h;
  Bin* b = bin_open(path, &st);
  if (!b) return st;
  if ((st = read_header(b, &h))) {
    bin_free(b);
    return st;
  }
  const int nb = h.num_baselines, nc = h.num_channels, T = h.num_times;
  metrix[0] = metrix[1] = metrix[2] = -1e12;
  metrix[3] = metrix[4] = metrix[5] = 1e12;
  for (int i = 0; i < nb; i++) {
    blws[2 * i] = -1e12;
    blws[2 * i + 1] = 1e12;
  }
  int ntpb = 0, mtpb = 0;
  if ((st = bin_read(b, T_INT, G_HEADER, H_NUM_TAGS_PER_BLOCK, 0, 4, &ntpb)) ||
      (st = bin_read(b, T_INT, G_HEADER, H_MAX_TIMES_PER_BLOCK, 0, 4, &mtpb))) {
    bin_free(b);
    return st;
  }
  if (mtpb <= 0 || nb < 0 || nc < 0 || T < 0) {
    /* the reference divides by zero or sizes negative arrays here */
    bin_free(b);
    return ST_FORMAT_BAD;
  }
  const int nblocks = (T + mtpb - 1) / mtpb;
  const size_t ntb = (size_t)mtpb * nb;
  double* ut = (double*)malloc(ntb * 8);
  double* vt = (double*)malloc(ntb * 8);
  double* wt = (double*)malloc(ntb * 8);
  double* at = (double*)malloc(ntb * nc * 64);
  double* il = (double*)malloc((size_t)nc * 8);
  for (int blk = 0; blk < nblocks && !st; blk++) {
    /* the reference accepts any start below the chunk count (a negative one
       indexes before its arrays); only valid starts are taken here */
    if ((long long)blk * ntpb >= 0 && (long long)blk * ntpb < b->n) b->search = blk * ntpb;
    int dim[6] = {0, 0, 0, 0, 0, 0};
    double fr[2], tr[2];
    if ((st = bin_read(b, T_INT, G_BLOCK, B_DIM_START_AND_SIZE, blk, 24, dim))) break;
    if ((st = bin_read(b, T_DOUBLE, G_BLOCK, B_FREQ_REF_INC_HZ, blk, 16, fr))) break;
    if ((st = bin_read(b, T_DOUBLE, G_BLOCK, B_TIME_REF_INC_MJD, blk, 16, tr))) break;
    double f = fr[0];
    for (int c = 0; c < nc; c++, f += fr[1]) il[c] = f / ORC_C_LIGHT;
    const int t0 = dim[0], c0 = dim[1], nt = dim[2];
    size_t ga, gu, gv, gw;
    if ((st = bin_read_n(b, T_DOUBLE | T_COMPLEX | T_MATRIX, G_BLOCK, B_CROSS_CORR, blk,
                         ntb * nc * 64, at, &ga)))
      break;
    if ((st = bin_read_n(b, T_DOUBLE, G_BLOCK, B_UU, blk, ntb * 8, ut, &gu))) break;
    if ((st = bin_read_n(b, T_DOUBLE, G_BLOCK, B_VV, blk, ntb * 8, vt, &gv))) break;
    if ((st = bin_read_n(b, T_DOUBLE, G_BLOCK, B_WW, blk, ntb * 8, wt, &gw))) break;
    /* Blocks that would make the reference write outside its outputs or read
       past the data it just read (undefined behaviour there) are rejected. */
    if (nt < 0 || nt > mtpb || t0 < 0 || t0 + nt > T || c0 != 0 ||
        ga < (size_t)nt * nb * nc * 64 || gu < (size_t)nt * nb * 8 ||
        gv < (size_t)nt * nb * 8 || gw < (size_t)nt * nb * 8) {
      st = ST_FORMAT_BAD;
      break;
    }
    for (int t = 0; t < nt; t++) {
      const int tt = t0 + t;
      for (int c = 0; c < nc; c++) {
        const int ct = c0 + c;
        for (int bl = 0; bl < nb; bl++) {
          const size_t i = 8 * ((size_t)bl + (size_t)nb * ((size_t)c + (size_t)nc * t));
          const size_t j = (size_t)bl + (size_t)nb * t;
          const double u = ut[j] * il[c], v = vt[j] * il[c], w = wt[j] * il[c];
          const size_t p = ((size_t)T * bl + tt) * nc + ct;
          uvws[3 * p] = u;
          uvws[3 * p + 1] = v;
          uvws[3 * p + 2] = w;
          metrix[0] = dmax(metrix[0], u);
          metrix[1] = dmax(metrix[1], v);
          metrix[2] = dmax(metrix[2], w);
          metrix[3] = dmin(metrix[3], u);
          metrix[4] = dmin(metrix[4], v);
          metrix[5] = dmin(metrix[5], w);
          blws[2 * bl] = dmax(blws[2 * bl], w);
          blws[2 * bl + 1] = dmin(blws[2 * bl + 1], w);
          memcpy(amps + 8 * p, at + i, 64);
        }
      }
    }
  }
  free(ut);
  free(vt);
  free(wt);
  free(at);
  free(il);
  bin_free(b);
  return st;
}

/* ------------------------------------------------------------------ writer */
typedef struct {
  int num_stations, num_times, num_channels, max_times_per_block;
  int amp_type;          /* type code stored in the AMP_TYPE header tag */
  int write_autocorr;    /* also write (zero) AUTO_CORRELATIONS per block */
  int trim_last_block;   /* last block's arrays hold only its own times */
  int extended_tags;     /* add named (extended) tags to the header and blocks */
  double freq_start_hz, freq_inc_hz, channel_bandwidth_hz, time_start_mjd_utc, time_inc_sec,
      time_average_sec;
  double phase_centre[2], telescope_centre[3];
} orc_vis_layout;

static int put_chunk(FILE* f, int type, int group, int tag, int user, const char* gname,
                     const char* tname, const void* data, size_t bytes) {
  uint8_t t[20];
  int es = (type & T_CHAR) ? 1 : (type & T_INT) ? 4 : (type & T_SINGLE) ? 4 : 8;
  if (type & T_COMPLEX) es *= 2;
  if (type & T_MATRIX) es *= 4;
  const int ext = gname != NULL;
  const size_t lg = ext ? strlen(gname) + 1 : 0, lt = ext ? strlen(tname) + 1 : 0;
  const uint64_t block = (uint64_t)bytes + lg + lt + 4;
  t[0] = 'T';
  t[1] = 0x42;
  t[2] = 'G';
  t[3] = (uint8_t)es;
  t[4] = (uint8_t)(0x40 | (ext ? 0x80 : 0));
  t[5] = (uint8_t)type;
  t[6] = (uint8_t)(ext ? lg : (size_t)group);
  t[7] = (uint8_t)(ext ? lt : (size_t)tag);
  for (int k = 0; k < 4; k++) t[8 + k] = (uint8_t)((uint32_t)user >> (8 * k));
  for (int k = 0; k < 8; k++) t[12 + k] = (uint8_t)(block >> (8 * k));
  uint32_t crc = orc_crc32c(t, 20);
  if (ext) {
    crc = crc_update(crc, gname, lg);
    crc = crc_update(crc, tname, lt);
  }
  crc = crc_update(crc, data, bytes);
  uint8_t cb[4] = {(uint8_t)crc, (uint8_t)(crc >> 8), (uint8_t)(crc >> 16),
                   (uint8_t)(crc >> 24)};
  if (fwrite(t, 20, 1, f) != 1) return ST_WRITE_FAIL;
  if (ext && (fwrite(gname, lg, 1, f) != 1 || fwrite(tname, lt, 1, f) != 1))
    return ST_WRITE_FAIL;
  if (bytes && fwrite(data, 1, bytes, f) != bytes) return ST_WRITE_FAIL;
  if (fwrite(cb, 4, 1, f) != 1) return ST_WRITE_FAIL;
  return 0;
}

#define PUT(type, group, tag, user, data, bytes)                                   \
  do {                                                                             \
    if ((st = put_chunk(f, type, group, tag, user, NULL, NULL, data, bytes))) goto out; \
  } while (0)

/* amps: [T][C][B][8] doubles (4 complex polarisations), uu/vv/ww: [T][B] metres. */
int orc_oskar_write(const char* path, const orc_vis_layout* L, const double* amps,
                    const double* uu, const double* vv, const double* ww) {
  const int S = L->num_stations, T = L->num_times, C = L->num_channels;
  const int M = L->max_times_per_block, B = S * (S - 1) / 2;
  const int nblocks = (T + M - 1) / M;
  const int ntpb = 7 + (L->write_autocorr ? 1 : 0) + (L->extended_tags ? 1 : 0);
  int st = 0;
  FILE* f = fopen(path, "wb");
  if (!f) return ST_OPEN_FAIL;
  double* blk_a = (double*)calloc((size_t)M * C * B * 8, 8);
  double* blk_u = (double*)calloc((size_t)M * B * 3, 8);
  double* auto_a = L->write_autocorr ? (double*)calloc((size_t)M * C * S * 8, 8) : NULL;
  double* stat = (double*)calloc((size_t)S, 8);
  uint8_t hdr[64];
  memset(hdr, 0, 64);
  memcpy(hdr, "OSKARBIN", 8);
  hdr[9] = 2;
  if (fwrite(hdr, 64, 1, f) != 1) {
    st = ST_WRITE_FAIL;
    goto out;
  }
  {
    const char tel[] = "synthetic.tm";
    const int wa = L->write_autocorr;
    PUT(T_CHAR, G_HEADER, H_TELESCOPE_PATH, 0, tel, sizeof(tel));
    PUT(T_INT, G_HEADER, H_NUM_TAGS_PER_BLOCK, 0, &ntpb, 4);
    PUT(T_INT, G_HEADER, H_WRITE_AUTOCORR, 0, &wa, 4);
    PUT(T_INT, G_HEADER, H_AMP_TYPE, 0, &L->amp_type, 4);
    PUT(T_INT, G_HEADER, H_MAX_TIMES_PER_BLOCK, 0, &M, 4);
    PUT(T_INT, G_HEADER, H_NUM_TIMES_TOTAL, 0, &T, 4);
    PUT(T_INT, G_HEADER, H_NUM_CHANNELS, 0, &C, 4);
    PUT(T_INT, G_HEADER, H_NUM_STATIONS, 0, &S, 4);
    PUT(T_DOUBLE, G_HEADER, H_FREQ_START_HZ, 0, &L->freq_start_hz, 8);
    PUT(T_DOUBLE, G_HEADER, H_FREQ_INC_HZ, 0, &L->freq_inc_hz, 8);
    PUT(T_DOUBLE, G_HEADER, H_CHANNEL_BW_HZ, 0, &L->channel_bandwidth_hz, 8);
    PUT(T_DOUBLE, G_HEADER, H_TIME_START_MJD, 0, &L->time_start_mjd_utc, 8);
    PUT(T_DOUBLE, G_HEADER, H_TIME_INC_SEC, 0, &L->time_inc_sec, 8);
    PUT(T_DOUBLE, G_HEADER, H_TIME_AVERAGE_SEC, 0, &L->time_average_sec, 8);
    PUT(T_DOUBLE, G_HEADER, H_PHASE_CENTRE, 0, L->phase_centre, 16);
    PUT(T_DOUBLE, G_HEADER, H_TELESCOPE_CENTRE, 0, L->telescope_centre, 24);
    PUT(T_DOUBLE, G_HEADER, H_STATION_X, 0, stat, (size_t)S * 8);
    PUT(T_DOUBLE, G_HEADER, H_STATION_Y, 0, stat, (size_t)S * 8);
    PUT(T_DOUBLE, G_HEADER, H_STATION_Z, 0, stat, (size_t)S * 8);
    if (L->extended_tags) {
      const int one = 1;
      if ((st = put_chunk(f, T_INT, 0, 0, 0, "rc_test", "header_note", &one, 4))) goto out;
    }
  }
  for (int blk = 0; blk < nblocks; blk++) {
    const int t0 = blk * M, nt = T - t0 < M ? T - t0 : M;
    const int rows = L->trim_last_block ? nt : M;
    const int dim[6] = {t0, 0, nt, C, B, S};
    const double fr[2] = {L->freq_start_hz, L->freq_inc_hz};
    const double tr[2] = {L->time_start_mjd_utc + t0 * L->time_inc_sec / 86400.0,
                          L->time_inc_sec / 86400.0};
    memset(blk_a, 0, (size_t)M * C * B * 64);
    memset(blk_u, 0, (size_t)M * B * 24);
    memcpy(blk_a, amps + (size_t)t0 * C * B * 8, (size_t)nt * C * B * 64);
    memcpy(blk_u, uu + (size_t)t0 * B, (size_t)nt * B * 8);
    memcpy(blk_u + (size_t)M * B, vv + (size_t)t0 * B, (size_t)nt * B * 8);
    memcpy(blk_u + (size_t)2 * M * B, ww + (size_t)t0 * B, (size_t)nt * B * 8);
    PUT(T_INT, G_BLOCK, B_DIM_START_AND_SIZE, blk, dim, 24);
    PUT(T_DOUBLE, G_BLOCK, B_FREQ_REF_INC_HZ, blk, fr, 16);
    PUT(T_DOUBLE, G_BLOCK, B_TIME_REF_INC_MJD, blk, tr, 16);
    if (L->write_autocorr)
      PUT(T_DOUBLE | T_COMPLEX | T_MATRIX, G_BLOCK, B_AUTO_CORR, blk, auto_a,
          (size_t)rows * C * S * 64);
    PUT(T_DOUBLE | T_COMPLEX | T_MATRIX, G_BLOCK, B_CROSS_CORR, blk, blk_a,
        (size_t)rows * C * B * 64);
    PUT(T_DOUBLE, G_BLOCK, B_UU, blk, blk_u, (size_t)rows * B * 8);
    PUT(T_DOUBLE, G_BLOCK, B_VV, blk, blk_u + (size_t)M * B, (size_t)rows * B * 8);
    PUT(T_DOUBLE, G_BLOCK, B_WW, blk, blk_u + (size_t)2 * M * B, (size_t)rows * B * 8);
    if (L->extended_tags) {
      if ((st = put_chunk(f, T_INT, 0, 0, blk, "rc_test", "block_note", &blk, 4))) goto out;
    }
  }
out:
  free(blk_a);
  free(blk_u);
  free(auto_a);
  free(stat);
  if (fclose(f) != 0 && !st) st = ST_WRITE_FAIL;
  return st;
}
