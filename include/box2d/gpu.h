/*
 * box2d/gpu.h -- additive entry points of the GB300 backend.
 *
 * None of these has a counterpart in the reference API: they expose what only a
 * device-resident implementation has (device status, device timers, the arena of a
 * world) and the batched and differentiable forms of b2World_Step.  The functions of
 * box2d.h keep their reference behaviour unchanged.
 */
#pragma once

#include "box2d.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Device status of a world: 0 when healthy, otherwise the CUDA error code of the first
 * failure.  A failed world stops stepping; the process is never aborted. */
B2_API int b2World_GetStatus( b2WorldId worldId );

/* Number of fast-body sweeps that reached a static candidate.  Time of impact is not
 * computed by this backend; a non-zero count means the step diverged from the reference
 * for those bodies. */
B2_API int b2World_GetUnsupportedToiCount( b2WorldId worldId );

/* Device stage timings of the last step (milliseconds, CUDA events on the world's
 * stream): whole step, narrowphase, solver (prepare .. store impulses), finalisation. */
typedef struct b2DeviceTimes
{
	float step; /* whole b2World_Step, host work included */
	float collide;
	float solve;
	float finalize;
	int eventCount;	 /* narrowphase begin/end/disjoint events */
	int recordCount; /* finalisation records (grown proxies, fast shapes) */
	int launches;	 /* kernel launches of the last step */
} b2DeviceTimes;

B2_API void b2World_EnableDeviceTiming( b2WorldId worldId, bool flag );
B2_API b2DeviceTimes b2World_GetDeviceTimes( b2WorldId worldId );

/* Copies p.x p.y q.c q.s v.x v.y w (7 floats) of every body id into out (7 * capacity
 * floats).  One device-to-host copy per call.  Returns the number of body ids. */
B2_API int b2World_GetBodyStates( b2WorldId worldId, float* out, int capacity );

#ifdef __cplusplus
}
#endif
