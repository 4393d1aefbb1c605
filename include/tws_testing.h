/* tws_testing.h -- test-only entry points of libtws.so.
 *
 * Not part of the drop-in interface (include/tws.h): an integrator has no use
 * for these, and including this header is a deliberate choice.  Nothing here
 * has a counterpart in the reference, whose shaders have no waits that can
 * run out.
 */
#ifndef TWS_TESTING_H
#define TWS_TESTING_H

#include "tws.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Failure-detection hook.  With drop = 1 every tile load of this grid's step
 * kernels arms its barrier for the tile's bytes but issues no copy, so each
 * bounded wait (tws_set_wait_limit) runs out with nothing in flight: the
 * kernel records the time-out and returns, and the next tws_sync or
 * tws_batch_sync reports TWS_ERR_TIMEOUT once.  drop = 0 turns it off.
 * Returns TWS_ERR_INVALID for other values. */
TWS_API int tws_test_drop_tile_loads(tws_grid* grid, int drop);

#ifdef __cplusplus
}
#endif

#endif /* TWS_TESTING_H */
