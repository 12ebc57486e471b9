/*
 * mrsr_test.h -- INTERNAL test hooks of libmrsr.so.  Not part of the product
 * ABI in mrsr.h: no reference method maps to these, and applications must not
 * call them.  They exist so the test suite can drive error-reporting paths
 * without provoking a device fault.
 */
#ifndef MRSR_TEST_H
#define MRSR_TEST_H

#include "mrsr.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Writes `code` into the operator's device error word (synchronous on
 * `stream`), as a kernel whose bounded wait gave up would.  The next
 * mrsr_normalop_check / CG call then reports MRSR_ERR_DEVICE. */
int mrsr_test_set_device_error(mrsr_normalop* op, int code, mrsr_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* MRSR_TEST_H */
