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

#ifdef __cplusplus
}
#endif

#endif /* HEU_GB300_PROBE_H_ */
