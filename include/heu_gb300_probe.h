/*
 * Measurement probe shipped with the engine library.  It has no counterpart
 * in the reference: it measures the device's integer multiply-accumulate
 * throughput, the denominator of the Montgomery kernels' roofline.
 */
#ifndef HEU_GB300_PROBE_H_
#define HEU_GB300_PROBE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* pattern 0: 32x32->64 MACs as mad.lo.cc/madc.hi.cc carry chains; pattern 1:
 * MACs as mad.wide.u32 into 64-bit accumulators (the device's fastest integer
 * MAC form, the roofline peak).  Returns 0 on success. */
int hg_probe_mac_peak(int device, int pattern, double* macs_per_second, double* seconds);

/* Number of engine kernels this process has launched so far. */
int hg_probe_launch_count(uint64_t* out);

/* Failure injection on the host: caps the device bytes the engine's buffers
 * may hold (0 = no cap).  A call whose buffers would pass the cap fails with
 * HG_ERR_NOMEM before any cudaMalloc; the context stays usable.  Reports
 * the bytes held now. */
int hg_probe_set_alloc_limit(size_t bytes, size_t* held_bytes);

/* How the engine's CUDA runtime sees a host pointer (the
 * cudaPointerAttributes type: 0 unregistered, 1 pinned host, 2 device,
 * 3 managed) and the bandwidth of one `bytes` copy between it and a fresh
 * device buffer on `device` (dir 0: host to device, 1: device to host). */
int hg_probe_host_copy(int device, void* host, size_t bytes, int dir, int* mem_type, double* gbs);

/* Open-loop load generator for the request server: Poisson arrivals at
 * `rate`/s, lengths log-uniform in [len_min, len_max], keys uniform over
 * key_ids, ops drawn with op_weights over (encrypt, add, mul, sum, decrypt);
 * add / mul / sum / decrypt read the key's resident vector handles[i],
 * encrypt reads m_host / r_host, mul reads k_host; every result goes to
 * `sink` (a timing sink, overwritten).  Fills latencies[nreq] (seconds),
 * ops and lens, and the wall time from the first arrival to the last
 * completion. */
typedef struct hg_server hg_server;
typedef struct {
  const int* key_ids;
  int nkeys;
  const uint64_t* handles;
  double rate;
  size_t nreq;
  size_t len_min, len_max;
  double op_weights[5];
  uint64_t seed;
  const void* m_host;
  const void* r_host;
  const void* k_host;
  void* sink;
  double* phases;  /* optional, 3 x nreq: per request the seconds from submission to
                      its first micro-batch, staging and launch of that batch, and from
                      the launch to completion (the last slice's batch retired) */
} hg_load_spec;
int hg_probe_serve_load(hg_server* s, const hg_load_spec* spec, double* latencies, int* ops, uint64_t* lens,
                        double* wall_s);

/* Per-batch trace of the request server.  enable != 0 clears the trace and
 * starts recording (records, cap ignored); enable == 0 stops recording,
 * sets *n to the number of records and copies up to `cap` of them.  A record
 * is 12 doubles: slot index, class (0 regular, 1 express, 2 slow express),
 * slices, elements, op mask (bit per op: 0 encrypt, 1 decrypt, 2 add, 3 mul,
 * 4 sum), the host times (seconds since the trace started) at which the
 * batch was formed, launched and retired, the GPU time (seconds since a
 * reference event recorded when the trace started) at which its stream began
 * the batch, and the milliseconds its stream spent on staged copies, on the
 * kernels and on the copies back. */
int hg_probe_server_trace(hg_server* s, int enable, double* records, size_t cap, size_t* n);

#ifdef __cplusplus
}
#endif

#endif /* HEU_GB300_PROBE_H_ */
