/*
 * hella_io.h -- the host-side data paths either side of the GB300 search:
 * the SIGPROC filterbank reader, the candidate file and coincidencer
 * formats, candidate clustering, per-channel flag statistics, and an
 * in-process header + data-block ring standing in for the PSRDADA buffer.
 * Reference counterparts (Coherent-All-Sky-Monitor/casm-hella):
 *   src/hella/src/sigproc.cpp:60-191          read_header, open_filterbank_file
 *   src/hella/src/peaks.cu:129-259             output_peaks (file and socket formats)
 *   src/apps/casm_hella_refactored.cu:708-716,757-761   flag statistics output
 *   src/hella/src/dada.cpp:16-88               DADA header + data unit, parse_dada_header
 * Every call returns a status (hella_status of hella_search.h); nothing exits
 * or throws.
 */
#ifndef HELLA_IO_H
#define HELLA_IO_H

#include <stddef.h>
#include <stdint.h>

#include "hella_search.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- SIGPROC filterbank (sigproc.cpp:60-191) */
/* Entries of a FREQUENCY_START table (the reference's frequency_table[4096],
 * sigproc.h:49); a file with more returns HELLA_ERR_INVALID_ARG, where the
 * reference writes past its array. */
#define HELLA_FIL_MAX_FREQ 4096
typedef struct {
  int machine_id, telescope_id, data_type, nchans, nbits, nifs, barycentric, pulsarcentric, ibeam, nbeams;
  double tstart, tsamp, fch1, foff, refdm, az_start, za_start, src_raj, src_dej, period;
  char isign;              /* "signed" */
  long npuls;
  char source_name[81], rawdatafile[81];
  int nfreq;               /* entries of a FREQUENCY_START table (fch1 = foff = 0 then) */
  long header_bytes;       /* offset of the first sample */
  double frequency_table[HELLA_FIL_MAX_FREQ]; /* the table's fchannel values, in file order
                                                 (hdr->frequency_table, sigproc.cpp:121-123) */
} hella_fil_header;

typedef struct hella_fil hella_fil;
/* Opens a filterbank file and parses its header.  expect_nchan > 0 checks
 * nchans against it (the reference's NCHAN check, :180-183); nbits must be 8
 * (:184-187).  HELLA_ERR_INVALID_ARG for a missing HEADER_START, an unknown
 * key or a failed check; HELLA_ERR_STATE for a truncated header. */
hella_status hella_fil_open(hella_fil **f, const char *path, int expect_nchan, hella_fil_header *hdr);
/* Reads up to nsamp spectra (u8 [nsamp][nchans]) into out; *got = spectra read. */
hella_status hella_fil_read(hella_fil *f, uint8_t *out, int nsamp, int *got);
void hella_fil_close(hella_fil *f);

/* ---- candidate output (peaks.cu:129-259) */
/* "SNR SAMP_START TIME_START WIDTH DM_IDX DM BEAM_IDX" */
#define HELLA_CAND_FILE_HEADER "SNR SAMP_START TIME_START WIDTH DM_IDX DM BEAM_IDX"
/* Lines "%g %d %g %d %d %g %d\n" of n candidates: snr, samp + samp0,
 * time_resolution * (samp + samp0) / 86400, width, dm_idx, dms[dm_idx],
 * beam (already offset by beam0).  *len = bytes written (no NUL counted);
 * HELLA_ERR_BUDGET when cap is too small (nothing is truncated silently). */
hella_status hella_cands_format(const hella_cand *c, int n, long samp0, const float *dms, int ndms,
                                double time_resolution, char *buf, size_t cap, size_t *len);
/* Appends the lines to the file at path, writing the header line first if
 * the file is empty (output_peaks' file branch). */
hella_status hella_cands_append(const char *path, const hella_cand *c, int n, long samp0, const float *dms,
                                int ndms, double time_resolution);
/* The coincidencer message (output_peaks' socket branch): a first line
 * "<gulp number>" (+ " UTC_START PICOSECONDS TSAMP" when utc_start is not
 * NULL, the DADA input case), then the candidate lines. */
hella_status hella_cands_coincidencer(int gulp_number, const char *utc_start, const char *picoseconds,
                                      const char *tsamp, const hella_cand *c, int n, long samp0,
                                      const float *dms, int ndms, double time_resolution, char *buf,
                                      size_t cap, size_t *len);

/* Sends len bytes of msg (e.g. a hella_cands_coincidencer message) over one
 * TCP connection to host (dotted IPv4) : port, then closes it (output_peaks'
 * socket branch, peaks.cu:179-258: connect, one message, close).  Partial
 * writes are continued until every byte is sent; the socket is closed on
 * every path.  timeout_ms > 0 bounds the connect and each write (0: the
 * system's blocking behaviour).  HELLA_ERR_INVALID_ARG for a bad host or
 * port, HELLA_ERR_IO when the connection or a write fails or times out. */
hella_status hella_cands_send(const char *host, int port, const char *msg, size_t len, int timeout_ms);

/* ---- candidate clustering (no counterpart in the reference) */
/* Friends-of-friends: two candidates of the same beam are friends when
 * |samp difference| <= dsamp, |dm_idx difference| <= ddm and |width
 * difference| <= dwidth; clusters are the connected components.  out gets
 * one representative per cluster (the highest snr, the earliest on ties), in
 * the order of their first member; labels (may be NULL) gets each input's
 * cluster index. */
hella_status hella_cluster(const hella_cand *in, int n, int dsamp, int ddm, int dwidth, hella_cand *out,
                           int *nout, int *labels);

/* ---- per-channel flag statistics (casm_hella_refactored.cu:708-716,757-761) */
/* The reference adds ntime x the cumulative d_flagSpec every searched gulp
 * (and that buffer is never zeroed); here each update adds ntime x this
 * gulp's increment of the cumulative fractions, so counts grow by what the
 * gulp flagged. */
typedef struct hella_flagstats hella_flagstats;
hella_status hella_flagstats_create(hella_flagstats **s, int nchan, int ntime);
void hella_flagstats_destroy(hella_flagstats *s);
/* cumulative[nchan]: hella_get_flag_spec / hella_batch_get_flag_spec. */
hella_status hella_flagstats_update(hella_flagstats *s, const float *cumulative);
hella_status hella_flagstats_counts(const hella_flagstats *s, long *counts);
/* Appends one "%d" line per channel (the specflags file). */
hella_status hella_flagstats_append(const hella_flagstats *s, const char *path);

/* ---- in-process header + data-block ring (dada.cpp:16-88) */
/* One writer and one reader in one process: the writer fills empty blocks,
 * the reader consumes filled blocks in order; a header block is written
 * once before the data.  pinned != 0 allocates the blocks page-locked
 * (cudaHostAlloc), so the search copies them to the GPU at full speed. */
typedef struct hella_ring hella_ring;
hella_status hella_ring_create(hella_ring **r, size_t block_bytes, int nblocks, int pinned);
void hella_ring_destroy(hella_ring *r);
size_t hella_ring_block_bytes(const hella_ring *r);
hella_status hella_ring_write_header(hella_ring *r, const char *header, size_t len);
/* Waits up to timeout_ms for the header; *len = its length (copied up to cap). */
hella_status hella_ring_read_header(hella_ring *r, char *out, size_t cap, size_t *len, int timeout_ms);
/* Writer: the next empty block (HELLA_ERR_TIMEOUT after timeout_ms), then
 * mark it filled with nbytes <= block_bytes.  hella_ring_end: no more data. */
hella_status hella_ring_open_write(hella_ring *r, uint8_t **block, int timeout_ms);
hella_status hella_ring_mark_filled(hella_ring *r, size_t nbytes);
hella_status hella_ring_end(hella_ring *r);
/* Reader: the next filled block (*nbytes = 0 and HELLA_OK at the end of the
 * data), then mark it cleared. */
hella_status hella_ring_open_read(hella_ring *r, const uint8_t **block, size_t *nbytes, int timeout_ms);
hella_status hella_ring_mark_cleared(hella_ring *r);
/* parse_dada_header (dada.cpp:50-79): "KEY value" lines up to the first NUL;
 * empty lines skipped; a line without a space ends the parse.  Copies the
 * value of `key` into val; HELLA_ERR_INVALID_ARG if it is absent. */
hella_status hella_header_get(const char *header, size_t len, const char *key, char *val, size_t cap);

#ifdef __cplusplus
}
#endif
#endif
