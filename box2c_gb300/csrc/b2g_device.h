/*
 * b2g_device.h -- C interface between the host step driver (C) and the CUDA side
 * (device arena management, transfers and kernel launch sequences).
 */
#pragma once

#include "b2g_types.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Colour-major layout of one step's constraint rows and joint list.  Colour c (0..10)
 * owns rows [colorStart[c], colorStart[c+1]) and joints [jointStart[c], jointStart[c+1]);
 * colour 11 is the overflow set, solved serially in list order. */
/* CTAs of the fused solver's thread-block cluster; body id b belongs to CTA
 * b / bodyBlock. */
#define B2G_FUSED_CTAS 16

typedef struct b2gSolvePlan
{
	int colorStart[B2G_COLORS + 1];
	int jointStart[B2G_COLORS + 1];
	int active[B2G_COLORS];
	int activeCount;
	int awakeCount;
	int bodyIdCount; /* body ids in use (0: caller buffers, per-phase kernels only) */
	/* Within colour c (< 11) the rows are grouped by the CTA owning their first
	 * non-static body: rowSplit[c][o] rows for CTA o, in CTA order.  bodyBlock = 0 means
	 * no grouping (the fused solver is not used). */
	int bodyBlock;
	int rowSplit[B2G_OVERFLOW][B2G_FUSED_CTAS];
} b2gSolvePlan;

/* Pinned host staging owned by the device module (mapped into the device). */
typedef struct b2gHostIO
{
	int* counters;		/* [0] events [1] records [2] status [3] sleepy bodies, copied back each sync */
	int* events;		/* mapped: narrowphase events */
	b2gRecord* records; /* mapped: finalisation records */
	int* sleepy;		/* mapped: bodies past the sleep time, 2 ints each (awake index, sleep time bits) */
	b2gContactInit* newContacts;
	int* hitIds;	/* mapped: contacts to test for hit events */
	float* hitOut; /* mapped: 8 per contact: hit, approach speed, point, normal, 0, 0 */
	int hitCap;
} b2gHostIO;

/* Host memory of the library through the caller's allocator (util.c). */
void* b2g_calloc( size_t count, size_t size );
void b2g_free( void* p );

int b2gd_device_ok( void );
const char* b2gd_last_error( void );

int b2gd_init( b2gDevWorld* w, b2gHostIO* io );
void b2gd_free( b2gDevWorld* w, b2gHostIO* io );

/* Grow device arrays (contents preserved). Returns 0 on success. */
int b2gd_reserve( b2gDevWorld* w, b2gHostIO* io, int bodyCap, int shapeCap, int contactCap, int jointCap, int solveCap,
				  int listCap );

/* Host -> device copies of body / shape / list data (host arrays use the device layout). */
int b2gd_upload_bodies( b2gDevWorld* w, const float* state, const float* xf, const float* centers, const float* prev,
						const float* mass, const float* force, const float* extent, const int* info, int count );
int b2gd_upload_awake( b2gDevWorld* w, const int* awake, int count );
/* Sleep timers and the mapped list of bodies past the sleep time for every body (worlds
 * that step with sleep on; elsewhere neither exists and finalisation skips the timers). */
int b2gd_reserve_sleep( b2gDevWorld* w, b2gHostIO* io );
int b2gd_reserve_body_ops( b2gDevWorld* w, int count );
/* Applies ops[0, count) (one per body, (bodyId << 2) | B2G_BODY_*) on the world's stream
 * (sleep: stop integrating; wake: identity state, zero sleep timer).  The copy is taken
 * from pageable memory, so ops may be reused when the call returns. */
int b2gd_body_ops( b2gDevWorld* w, const int* ops, int count );
int b2gd_upload_shapes( b2gDevWorld* w, const b2gShapeGeo* geo, const float* aabb, const float* fat, int count );
int b2gd_upload_shape_lists( b2gDevWorld* w, const int* range, int bodyCount, const int* list, int listCount );
int b2gd_upload_joints( b2gDevWorld* w, const b2gJointDev* joints, int count );
int b2gd_upload_solve_lists( b2gDevWorld* w, const int* solveList, int solveCount, const int* jointList, int jointCount );
int b2gd_upload_fat( b2gDevWorld* w, int shapeId, const float* fat4 );
int b2gd_upload_body_velocity( b2gDevWorld* w, int bodyId, const float* v3 );
/* Pose of one body after a time-of-impact event: transform, centre (with local centre)
 * and sweep start; tight and fat boxes of one of its shapes.  Stream-ordered copies. */
int b2gd_upload_pose( b2gDevWorld* w, int bodyId, const float* xf4, const float* center4, const float* prev4 );
int b2gd_upload_shape_boxes( b2gDevWorld* w, int shapeId, const float* aabb4, const float* fat4 );

/* Device -> host copies. */
int b2gd_download_bodies( b2gDevWorld* w, float* state, float* xf, float* centers, int count );
int b2gd_download_manifolds( b2gDevWorld* w, b2gManifold* out, uint32_t* flags, int count );
/* Hit test of the contacts ids[0..n) after the solver stage (reference
 * src/solver.c:1670-1723): out[8 k ..] = hit flag, approach speed and point of the
 * fastest approaching point above `threshold` with a positive impulse, then the normal.
 * Synchronises the world's stream; ids and results are io->hitIds / io->hitOut. */
int b2gd_hit_events( b2gDevWorld* w, b2gHostIO* io, int n, float threshold );
int b2gd_reserve_hits( b2gHostIO* io, int n );
int b2gd_download_shapes( b2gDevWorld* w, float* aabb, float* fat, int count );
int b2gd_download_joints( b2gDevWorld* w, b2gJointDev* joints, int count );

/* Step stages.  b2gd_collide launches contact creation and the narrowphase and copies
 * the event count back; b2gd_solve launches the solver and finalisation and copies the
 * record count back.  b2gd_sync waits for the stream; returns 0 or a CUDA error. */
int b2gd_collide( b2gDevWorld* w, b2gHostIO* io, int newContactCount, int contactIdCount );
int b2gd_solve( b2gDevWorld* w, b2gHostIO* io, const b2gSolvePlan* plan, const b2gStepConst* sc );
/* The fused solver stage and finalisation launched before the narrowphase's events are
 * known; they do nothing when there were events.  1 launched, 0 not (the world does not
 * fit the fused solver), -1 launch error. */
int b2gd_solve_speculative( b2gDevWorld* w, b2gHostIO* io, const b2gSolvePlan* plan, const b2gStepConst* sc );
int b2gd_sync( b2gDevWorld* w );

/* ---------------------------------------------------------------- broadphase query */
/* Device pair query of one step's moved proxies (reference src/broad_phase.c:278-331
 * b2FindPairsTask): for each moved proxy key (proxyId << 2 | tree type, or B2G_NULL), the
 * leaves of the kinematic, static (dynamic proxies only) and dynamic trees whose fat
 * boxes overlap its fat box, in the order of the host tree query (depth first, child1
 * pushed before child2).  Candidates of proxy i are cand[2 * (B2G_QUERY_SLOTS * i + k)]
 * (leaf proxy key) and cand[... + 1] (shape id) for k < counts[i]; counts[i] is -1 when
 * the proxy needed more than B2G_QUERY_SLOTS slots or a deeper stack, and the host
 * queries that proxy itself.  Candidates the pair rules reject for the proxy itself, the
 * moved-pair rule or an existing pair (pairTable: the host pair set's table of pairCap
 * slots, copied when pairVersion changes) are left out.  Synchronises the world's
 * stream; the result arrays are host memory owned by the query and valid until the next
 * call. */
#define B2G_QUERY_SLOTS 32

typedef struct b2gPairQuery b2gPairQuery;

int b2gd_pair_query( b2gDevWorld* w, b2gPairQuery** query, const b2gTreeNode* const nodes[3], const int capacity[3], const int root[3],
					 const int* keys, int count, const unsigned long long* pairTable, int pairCap, unsigned pairVersion,
					 const int** cand, const int** counts );
void b2gd_pair_query_free( b2gPairQuery* query );

/* ---------------------------------------------------------------- batched worlds */
/* One world of a batched step (device copy of its descriptor plus the step's counts).
 * W.counters points into the batch's counter array, 4 ints per world. */
typedef struct b2gBatchItem
{
	b2gDevWorld W;
	b2gStepConst sc;
	int colorStart[B2G_COLORS + 1];
	int jointStart[B2G_COLORS + 1];
	int active[B2G_COLORS];
	int activeCount;
	int awakeCount;
	int bodyIdCount;
	int idCount; /* contact ids run through the narrowphase */
	int staged;	 /* staged contact records */
	int solve;	 /* 1 when the solver stage runs */
	int tapeRows;	  /* rows recorded for the adjoint this step */
	void* tapeBodies; /* adjoint tape destinations, or null when not recording */
	void* tapeRowDst;
	int widest;		/* most rows + joints of any colour but the overflow colour */
	int rowsOnChip; /* 1 when the solver keeps this world's rows in shared memory (set at launch) */
} b2gBatchItem;

/* Device context of batched steps: pinned staging of items and counters, device copies,
 * captured CUDA graphs and the solver autotuner's state. */
typedef struct b2gBatch b2gBatch;

b2gBatch* b2gd_batch_create( void );
void b2gd_batch_destroy( b2gBatch* b );
/* Grows the item and counter buffers; returns the pinned item array or null. */
b2gBatchItem* b2gd_batch_items( b2gBatch* b, int count );
void* b2gd_batch_stream( b2gBatch* b );
/* Worlds with more body ids than this are stepped alone (b2World_Step) by the batch. */
int b2gd_batch_max_bodies( void );
/* Host copy of world i's 4 counters after the last sync. */
const int* b2gd_batch_counters( b2gBatch* b, int i );
/* A step's items run in halves (h = 0, 1: items [first, first + count)), each with its
 * own graphs, so that the host phases of one half overlap the device work of the other;
 * everything is ordered on the batch's stream.  begin_step picks the solver's launch
 * shape for the step; end_step waits for the stream and does the timing and tuning. */
void b2gd_batch_begin_step( b2gBatch* b );
/* Narrowphase of a half (contact records staged by b2gd_stage_contacts). */
int b2gd_batch_collide( b2gBatch* b, int h, int first, int count );
/* Solver stage and finalisation of a half's items with solve != 0: packs of
 * similar-sized worlds, each world on one warp, a group of warps or a whole CTA. */
int b2gd_batch_solve( b2gBatch* b, int h, int first, int count );
int b2gd_batch_wait_collide( b2gBatch* b, int h );
int b2gd_batch_wait_solve( b2gBatch* b, int h );
int b2gd_batch_end_step( b2gBatch* b );
/* Device milliseconds of the last batched narrowphase and solve, the solver's CTA size
 * and resident CTAs per SM, and the number of kernel launches. */
void b2gd_batch_stats( b2gBatch* b, float* collideMs, float* solveMs, int* threads, int* ctasPerSm, int* launches );
/* Copies a world's staged contact records to the device on the world's stream. */
int b2gd_stage_contacts( b2gDevWorld* w, b2gHostIO* io, int count );

/* ---------------------------------------------------------------- step adjoint */
/* One solver row as recorded for the adjoint: the contact, its bodies (-1 static) and
 * shapes, mixed material and the manifold the solver stage starts from. */
typedef struct b2gTapeRow
{
	int32_t cid, ia, ib, shapeA, shapeB, pad;
	float friction, restitution;
	b2gManifold m;
	float pad2[1];
} b2gTapeRow;

/* One recorded step: where its body and row records are in the world's tape, the
 * solve plan and the step constants. */
typedef struct b2gTapeStep
{
	int64_t bodyOff, rowOff; /* float4 offsets of the body records, b2gTapeRow offsets */
	int32_t bodies, rows, solve, pad;
	int32_t colorStart[B2G_COLORS + 1];
	int32_t jointStart[B2G_COLORS + 1];
	int32_t active[B2G_COLORS];
	int32_t activeCount, awakeCount;
	b2gStepConst sc;
} b2gTapeStep;

/* Body record: 4 float4 per body id: v.x v.y w tag | p.x p.y q.c q.s |
 * c.x c.y lc.x lc.y | awake 0 0 0. */
#define B2G_TAPE_BODY_FLOAT4 4

/* Records one step's solver inputs into the tape (world stream). */
int b2gd_tape_record( b2gDevWorld* w, void* bodyDst, int bodies, void* rowDst, int rows );

/* One world of a backward pass. */
typedef struct b2gAdjointItem
{
	b2gDevWorld W;			   /* geometry, mass, forces, damping of the world */
	const float* tapeBodies;   /* tape base (4 floats per float4 unit) */
	const b2gTapeRow* tapeRows; /* tape rows base */
	const b2gTapeStep* steps;  /* device copy of the step headers */
	int stepCount;
	int bodies;				   /* body ids (constant over the tape) */
	int shapes;
	int maxRows;
	int contactCap;
	int pad;
	const float* shapeFriction; /* per shape id */
	const float* gradFinal;		/* 6 per body id: p.x p.y angle v.x v.y w */
	float* gradInitial;			/* 6 per body id */
	float* gradFriction;		/* per shape id */
	float* scratch;
	int* status; /* [0] unsupported rows, [1] manifold replay mismatches */
} b2gAdjointItem;

/* Scratch floats one world needs for a backward pass. */
size_t b2gd_adjoint_scratch( int bodies, int maxRows, int contactCap, int subSteps );
/* Runs the backward pass of `count` worlds (device item array, one CTA each). */
int b2gd_adjoint_launch( const b2gAdjointItem* dItems, int count, void* stream );

/* Device time of the last step's stages in milliseconds (CUDA events recorded when
 * w->timing is set). */
void b2gd_enable_timing( b2gDevWorld* w, int flag );
void b2gd_stage_times( b2gDevWorld* w, float* stepMs, float* collideMs, float* solveMs, float* finalizeMs );
/* Records timer slot 0 (step start) or 6 (step end) on the world's stream. */
void b2gd_mark( b2gDevWorld* w, int slot );

#ifdef __cplusplus
}
#endif
