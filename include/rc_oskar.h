/*
 * rc_gb300 — OSKAR 2.6 visibility-file ingest (librc_gb300.so).
 *
 * 1. Drop-in symbols of the reference's OSKAR reader
 *    (SKA-ScienceDataProcessor/RC, MS6/kernel/oskar/OskarBinReader.h:34-78,
 *    bound from Haskell in MS6/kernel/oskar/OskarBinReaderFFI.hsc:54-67 and
 *    OskarReader.hs:40): the same names, struct layouts, argument meaning,
 *    output layouts and status codes.  The file's payloads are read by
 *    parallel host threads into pinned buffers, copied to the GPU, checked
 *    (CRC-32C) and reshuffled there, and copied back into the caller's host
 *    arrays.
 *
 * 2. Device entries (gb_oskar_*): the same read with the outputs left in
 *    device memory, and the pipeline's extraction of one channel and
 *    polarisation as 5-double records (MS6/programs/Kernel/IO.hs:22-74) or
 *    as uvw + complex visibilities for the gridding engine.
 *
 * Status codes: 0 on success; the container's negative codes below; the
 * reader's 0xdeadbeef for a file whose amplitudes are not double precision;
 * the GB_ERR_* codes of rc_gb300.h for argument, CUDA and allocation errors.
 * gb_last_error() gives the message.
 */
#ifndef RC_OSKAR_H
#define RC_OSKAR_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* u,v,w are stored in metres; u,v,w in wavelengths = metres * f / c. */
#ifndef SPEED_OF_LIGHT
#define SPEED_OF_LIGHT 299792458.0
#endif

/* Container status codes (MS6/kernel/oskar/oskar_binary/oskar_binary.h:96-114). */
#define GB_OSKAR_OPEN_FAIL (-100)
#define GB_OSKAR_SEEK_FAIL (-101)
#define GB_OSKAR_READ_FAIL (-102)
#define GB_OSKAR_FILE_INVALID (-106)
#define GB_OSKAR_FORMAT_BAD (-107)
#define GB_OSKAR_ENDIAN_MISMATCH (-108)
#define GB_OSKAR_VERSION_UNKNOWN (-109)
#define GB_OSKAR_TYPE_UNKNOWN (-110)
#define GB_OSKAR_INT_UNKNOWN (-111)
#define GB_OSKAR_FLOAT_UNKNOWN (-112)
#define GB_OSKAR_DOUBLE_UNKNOWN (-113)
#define GB_OSKAR_MEMORY_NOT_ALLOCATED (-114)
#define GB_OSKAR_TAG_NOT_FOUND (-115)
#define GB_OSKAR_CRC_FAIL (-118)
/* MS6/kernel/oskar/OskarBinReader.cpp:183-186: amplitudes not double. */
#define GB_OSKAR_NOT_DOUBLE ((int)0xdeadbeefu)

/* Opaque handle of an open file (the reference's oskar_Binary*). */
#ifndef OSKAR_BINARY_H_
struct oskar_Binary;
typedef struct oskar_Binary oskar_Binary;
#endif

/* MS6/kernel/oskar/OskarBinReader.h:34-52 — field order and types kept
 * because the Haskell side reads the counts at their C offsets. */
typedef struct VisData_tag {
  oskar_Binary *h;
  int num_baselines, num_channels, num_stations, num_times, num_times_baselines, num_points;
  double phase_centre[2], telescope_centre[3], freq_start_inc[2], time_start_inc[2],
      channel_bandwidth_hz, time_average_sec;
} VisData;

/* OskarBinReader.h:55-64 */
typedef struct Metrix_tag {
  double maxu, maxv, maxw, minu, minv, minw;
} Metrix;

/* OskarBinReader.h:67-72 (one per baseline) */
typedef struct WMaxMin_tag {
  double maxw, minw;
} WMaxMin;

/* Replaces mkFromFile (OskarBinReader.cpp:149-238): opens the file, indexes
 * its chunks and fills the header fields; vdp->h stays open until
 * freeBinHandler.  num_baselines = S(S-1)/2 for S stations, num_points =
 * times x baselines x channels. */
int mkFromFile(VisData *vdp, const char *filename);

/* Replaces freeBinHandler (OskarBinReader.cpp:240-242). */
void freeBinHandler(VisData *vdp);

/* Replaces readAndReshuffle (OskarBinReader.cpp:246-413).  Host outputs:
 *   amps  num_points x 4 complex doubles, [baseline][time][channel][pol]
 *   uvws  num_points x 3 doubles (wavelengths), [baseline][time][channel][uvw]
 *   mp    u/v/w extrema over all points (start values -1e12 / 1e12)
 *   bl_ws per-baseline w extrema (num_baselines entries).
 * Wavelength scale of channel c in a block: f_c / c with f_0 the block's
 * reference frequency and f_{c+1} = f_c + increment (repeated addition). */
int readAndReshuffle(const VisData *vdp, double *amps, double *uvws, Metrix *mp,
                     WMaxMin *bl_ws);

/* Replaces _aligned_malloc (OskarBinReader.cpp:38-48), which the reference
 * exports for its Haskell reader (OskarReader.hs:40): posix_memalign, NULL on
 * failure; release with free(). */
void *_aligned_malloc(size_t size, size_t alignment);

/* readAndReshuffle with device outputs: d_amps (num_points x 8 doubles) and
 * d_uvws (num_points x 3 doubles) are device pointers; mp and bl_ws are host
 * pointers (bl_ws may be NULL).  Synchronous: returns when the outputs are
 * complete on `stream` and every payload's CRC-32C has been checked. */
int gb_oskar_read_device(const VisData *vdp, double *d_amps, double *d_uvws, Metrix *mp,
                         WMaxMin *bl_ws, void *stream);

/* Timings of the calling thread's last readAndReshuffle / gb_oskar_read_device:
 * out4 = {host staging ms (parallel pread + copies to the device, wall
 * clock), CRC-32C kernel ms, reshuffle kernel ms (CUDA events on the read's
 * stream), whole call ms (wall clock)}.  The reference has no counterpart. */
int gb_oskar_last_timings(double *out4);

/* MS6/programs/Kernel/IO.hs:22-74 on the device: 5-double records
 * (u, v, w, re, im) of points [dom_low, dom_high) in [baseline][time] order
 * for channel `freq` and polarisation `pol`, from gb_oskar_read_device's
 * outputs.  dom_low must be a multiple of num_times (baseline-aligned), as
 * there.  flags & GB_OSKAR_REFERENCE_UVW_INDEX takes u,v,w from the address
 * that kernel uses, 3 * (time + num_times * baseline), which ignores the
 * channel stride (the same point only in single-channel files); without it
 * the point's own channel is used.  Needs only vdp's counts (the file may be
 * closed). */
#define GB_OSKAR_REFERENCE_UVW_INDEX 1
int gb_oskar_records(const VisData *vdp, const double *d_amps, const double *d_uvws,
                     int32_t freq, int32_t pol, int64_t dom_low, int64_t dom_high,
                     int32_t flags, double *d_records, void *stream);

/* One channel and polarisation of every point, [baseline][time] order, in the
 * gridding engine's input form: d_uvw (n x 3 doubles, wavelengths) and d_vis
 * (n complex values: complex64 when vis_f64 == 0, complex128 otherwise),
 * n = num_times_baselines.  Needs only vdp's counts.  Asynchronous on
 * `stream`. */
int gb_oskar_extract(const VisData *vdp, const double *d_amps, const double *d_uvws,
                     int32_t freq, int32_t pol, double *d_uvw, void *d_vis, int32_t vis_f64,
                     void *stream);

/* CRC-32C of n device bytes continued from a finished code `code` the way
 * the container does (0xFFFFFFFF = start; MS6/kernel/oskar/oskar_binary/src/
 * oskar_crc.c:109-160), computed on the GPU.  d_data must be 16-byte
 * aligned.  Synchronous. */
int gb_crc32c_device(const void *d_data, int64_t n, uint32_t code, uint32_t *out, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* RC_OSKAR_H */
