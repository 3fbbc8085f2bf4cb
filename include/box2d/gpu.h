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

/* Status of a world: 0 when healthy, otherwise the first failure: a CUDA error code
 * (positive), B2_STATUS_OUT_OF_HOST_MEMORY when the host allocator (b2SetAllocator, or
 * aligned_alloc by default) refused a request during a call on the world, or -1 for a
 * failed launch.  A failed world stops stepping; the process is never aborted.  Host
 * memory failures are counted process-wide, so a world worked on while another thread's
 * request failed is marked failed too. */
#define B2_STATUS_OUT_OF_HOST_MEMORY ( -2 )
B2_API int b2World_GetStatus( b2WorldId worldId );

/* Number of time-of-impact events since the world was created: fast bodies (and
 * bullets) that continuous collision moved back along their sweep to the first contact
 * with a static shape (or, for a bullet, with any non-bullet shape), as the reference's
 * src/solver.c:787-1105 does. */
B2_API int b2World_GetToiEventCount( b2WorldId worldId );

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
	int fusedSolver; /* 1 when the last step's solver stage ran as one fused launch */
	/* bytes the last step moved between host and device: copies (setup changes, new
	 * contacts, solve lists, tree nodes, counters, time-of-impact poses) and device
	 * reads or writes of mapped host memory (events, records, pair candidates) */
	long long hostToDeviceBytes;
	long long deviceToHostBytes;
	/* host phases of the last step (milliseconds): tree walks of the moved proxies on the
	 * device with their round trip, pair rules, contact creation, narrowphase events
	 * (colouring), solve lists (build and upload), partial tree rebuild, finalisation
	 * records (proxy enlargement, move buffer) and continuous collision */
	float hostPairQuery;
	float hostPairRules;
	float hostContactCreate;
	float hostEvents;
	float hostSolveLists;
	float hostTreeRebuild;
	float hostRecords;
	float hostContinuous;
} b2DeviceTimes;

B2_API void b2World_EnableDeviceTiming( b2WorldId worldId, bool flag );
B2_API b2DeviceTimes b2World_GetDeviceTimes( b2WorldId worldId );

/* Solver-stage implementation: one fused launch of a 16-CTA cluster that keeps the
 * world's bodies and constraint rows in shared memory (the default; used whenever the
 * world fits, roughly 20k contacts), or one kernel launch per phase.  Both give
 * bit-identical results. */
B2_API void b2World_EnableFusedSolver( b2WorldId worldId, bool flag );

/* Steps `count` independent worlds by one b2World_Step each.  The device work of all of
 * them runs together, in two halves whose host work overlaps the other half's device
 * work: replayed CUDA graphs for contact creation and the narrowphase of every world,
 * and for the solver stage and finalisation (a persistent kernel over packs of
 * similar-sized worlds, each world on a warp, a group of warps or a whole CTA).  A world
 * with more bodies than the batched solver holds (about 6900) is stepped alone in the
 * same call.  Every world gets exactly the results b2World_Step would give it alone.
 * Invalid, failed or repeated ids are skipped.  Not thread-safe: one batch at a time
 * per process. */
B2_API void b2World_StepBatch( const b2WorldId* worldIds, int count, float timeStep, int subStepCount );

/* Device milliseconds of the last batched step's narrowphase and solver segments (both
 * halves), the solver CTA size and resident CTAs per SM picked by the autotuner (0 while
 * it is still timing candidates), the kernel launches of the last batched step, and its
 * host milliseconds per segment.  A step runs its worlds in two halves so that one
 * half's host work overlaps the other's device work; the segments are: preparation of
 * the first half; its narrowphase launch, the second half's preparation and launch and
 * the tree rebuilds; the narrowphase waits, events and solve lists and solver launches;
 * the solver waits and finalisation records; the end of the step.  Per-world host work
 * runs on hostThreads threads. */
typedef struct b2BatchStats
{
	float collide;
	float solve;
	int solveThreads;
	int launches;
	float hostBegin, hostCollide, hostMiddle, hostSolve, hostFinish;
	int hostThreads;
	int solveCtasPerSm;
} b2BatchStats;

B2_API b2BatchStats b2World_GetBatchStats( void );

/* Differentiable stepping.  b2World_BeginTape starts recording the world's next
 * maxSteps steps (0 stops and frees the recording); each recorded step keeps the
 * solver inputs of that step on the device.  b2World_StepBackward then returns the
 * gradient of a scalar loss L through all recorded steps, by a hand-written adjoint of
 * the substepped soft-step solver (reverse colour order, each step recomputed from its
 * record).  States are 6 floats per body id: p.x p.y angle v.x v.y w.
 *   gradFinal     dL/d(state after the last recorded step)      (6 x bodies)
 *   gradInitial   dL/d(state before the first recorded step)    (6 x bodies, out)
 *   gradFriction  dL/d(shape friction) per shape id             (shapes, out, may be null)
 * The discrete choices of each step (pairs, colours, contact features, active clamps)
 * are those of the recorded steps.  Supported: polygon, capsule and segment shapes
 * without joints or overflow-colour constraints, and steps without time-of-impact
 * events; otherwise B2_ADJOINT_UNSUPPORTED.
 * B2_ADJOINT_REPLAY_MISMATCH reports that the recomputed contact geometry differed from
 * the recorded one (the world changed after recording).  No counterpart in the
 * reference API. */
#define B2_ADJOINT_UNSUPPORTED ( -3 )
#define B2_ADJOINT_REPLAY_MISMATCH ( -4 )

B2_API void b2World_BeginTape( b2WorldId worldId, int maxSteps );
B2_API int b2World_GetTapeSteps( b2WorldId worldId );
B2_API int b2World_StepBackward( b2WorldId worldId, const float* gradFinal, float* gradInitial, float* gradFriction );

/* The backward pass of `count` recorded worlds in one launch (one warp per world).
 * Arrays are per world with fixed strides: gradFinal / gradInitial 6 * bodyStride
 * floats per world, gradFriction shapeStride floats per world. */
B2_API int b2World_StepBackwardBatch( const b2WorldId* worldIds, int count, int bodyStride, int shapeStride, const float* gradFinal,
									  float* gradInitial, float* gradFriction );

/* Self-check of the last backward call: recorded manifolds the backward pass did not
 * reproduce, and replayed steps that did not end bit for bit where the next recorded
 * step starts (both 0 when the adjoint differentiated exactly the recorded steps). */
B2_API void b2World_GetBackwardCheck( int* manifoldMismatches, int* replayMismatches );

/* Copies p.x p.y q.c q.s v.x v.y w (7 floats) of every body id into out (7 * capacity
 * floats).  One device-to-host copy per call.  Returns the number of body ids. */
B2_API int b2World_GetBodyStates( b2WorldId worldId, float* out, int capacity );

/* One soft-step contact solve on caller-owned device buffers: the solver stage of
 * b2World_Step (reference src/solver.c:559-731 and src/contact_solver.c) without the
 * broadphase, narrowphase, colouring or body finalisation.  The caller supplies
 * coloured contacts (no two contacts of one colour share a non-static body; colour 11
 * is the overflow set, solved serially in array order) and receives updated body
 * velocities, position/rotation deltas and accumulated impulses.  All pointers are
 * device pointers except colorStart; the call is asynchronous on `stream`. */
typedef struct b2ContactSolveDesc
{
	/* bodies, indexed by body index */
	float* states;			/* in/out, 8 per body: v.x v.y w (unused) dp.x dp.y dq.c dq.s */
	const float* massData;	/* 4 per body: mass invMass inertia invInertia */
	const float* forces;	/* 4 per body: force.x force.y torque gravityScale */
	const float* damping;	/* 4 per body: linearDamping angularDamping (2 unused) */
	const int* bodies;		/* bodyCount body indices integrated every substep */
	int bodyCount;

	/* contacts, colour-major */
	const int* contactBodies; /* 2 per contact: body index, -1 for a static body */
	const float* contactMix;  /* 2 per contact: friction, restitution */
	b2Manifold* manifolds;	  /* in: points, centre-relative anchors, separations and
							   * warm-start impulses; out: impulses, max impulse and
							   * relative normal velocity per point */
	int contactCount;
	int colorStart[13]; /* host ints; colorStart[12] == contactCount */

	/* step */
	float timeStep;
	int subStepCount;
	b2Vec2 gravity;
	float contactHertz, contactDampingRatio, contactPushout, restitutionThreshold;
	bool enableWarmStarting;
	void* stream; /* cudaStream_t; null for the default stream */
} b2ContactSolveDesc;

/* Returns 0, or a CUDA error code / -1 for invalid arguments.  Allocates its per-call
 * constraint rows (144 bytes per contact) with stream-ordered device allocation. */
B2_API int b2SolveContacts( const b2ContactSolveDesc* desc );

/* b2SolveContacts that allocates nothing; no counterpart in the reference API.  Its
 * constraint rows live in one fixed device array per device, compiled into the library:
 * B2_SOLVE_NOALLOC_MAX_CONTACTS rows of 144 bytes (2.25 MiB).  Same descriptor and
 * results as b2SolveContacts, and its return codes but for the allocation failures it
 * cannot have, plus (nothing launched in either case):
 *   B2_SOLVE_NOALLOC_TOO_LARGE     contactCount exceeds B2_SOLVE_NOALLOC_MAX_CONTACTS;
 *   B2_SOLVE_NOALLOC_DEVICE_LIMIT  the current device's ordinal is 64 or more (the
 *                                  address cache holds 64 devices).
 * - The first call on each device (with that device current) looks up the array's
 *   address, and again after the device's context was replaced (cudaDeviceReset); make
 *   such calls before any stream capture starts.
 * - Nothing in the array has to start at zero: every row is written before it is read.
 * - Calls that overlap on one device share the array and race: order them (one stream,
 *   or events between streams, and one host thread at a time). */
#define B2_SOLVE_NOALLOC_MAX_CONTACTS 16384
#define B2_SOLVE_NOALLOC_TOO_LARGE ( -2 )
#define B2_SOLVE_NOALLOC_DEVICE_LIMIT ( -3 )

B2_API int b2SolveContactsNoAlloc( const b2ContactSolveDesc* desc );

#ifdef __cplusplus
}
#endif
