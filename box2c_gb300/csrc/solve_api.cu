/*
 * solve_api.cu -- b2SolveContacts: the solver stage of b2World_Step on caller-owned
 * device buffers (declared in include/box2d/gpu.h).
 *
 * It builds a world descriptor over the caller's arrays (contacts in order, no joints)
 * and runs the same launch sequence as the world step's solver stage
 * (b2gd_contact_solver: prepare, substeps of integrate / warm start / solve / integrate
 * positions / relax, restitution, store impulses).  The constraint rows are per-call
 * scratch taken from the stream-ordered device allocator.
 */
#include "b2g_device.h"

#include "box2d/gpu.h"

#include <cuda_runtime.h>

#include <string.h>

static_assert( sizeof( b2gManifold ) == sizeof( b2Manifold ), "device manifold must have the b2Manifold layout" );
static_assert( sizeof( b2gPoint ) == sizeof( b2ManifoldPoint ), "device manifold point must have the b2ManifoldPoint layout" );

extern "C" int b2gd_contact_solver( b2gDevWorld* w, const b2gSolvePlan* plan, const b2gStepConst* sc );

static void make_soft( float hertz, float zeta, float h, float* out )
{
	if ( hertz == 0.0f )
	{
		out[0] = 0.0f;
		out[1] = 1.0f;
		out[2] = 0.0f;
		return;
	}
	float omega = 2.0f * B2G_PI * hertz;
	float a1 = 2.0f * zeta + h * omega;
	float a2 = h * omega * a1;
	float a3 = 1.0f / ( 1.0f + a2 );
	out[0] = omega / a1;
	out[1] = a2 * a3;
	out[2] = a3;
}

/* Validates the descriptor and fills the step constants, the colour plan and the
 * descriptor fields that point at caller memory.  Returns 0 or -1. */
extern "C" int b2gd_contact_desc( const b2ContactSolveDesc* d, b2gDevWorld* w, b2gSolvePlan* plan, b2gStepConst* sc )
{
	if ( d == nullptr || d->states == nullptr || d->massData == nullptr || d->forces == nullptr || d->damping == nullptr )
		return -1;
	if ( d->contactCount < 0 || d->bodyCount < 0 || d->timeStep <= 0.0f )
		return -1;
	if ( d->contactCount > 0 && ( d->contactBodies == nullptr || d->contactMix == nullptr || d->manifolds == nullptr ) )
		return -1;
	if ( d->bodyCount > 0 && d->bodies == nullptr )
		return -1;
	if ( d->colorStart[0] != 0 || d->colorStart[B2G_COLORS] != d->contactCount )
		return -1;
	for ( int c = 0; c < B2G_COLORS; ++c )
		if ( d->colorStart[c + 1] < d->colorStart[c] )
			return -1;

	memset( sc, 0, sizeof( *sc ) );
	sc->subSteps = d->subStepCount < 1 ? 1 : d->subStepCount;
	sc->dt = d->timeStep;
	sc->inv_dt = 1.0f / d->timeStep;
	sc->h = d->timeStep / (float)sc->subSteps;
	sc->inv_h = (float)sc->subSteps * sc->inv_dt;
	float contactHertz = gmin( d->contactHertz, 0.25f * sc->inv_h );
	make_soft( contactHertz, d->contactDampingRatio, sc->h, sc->contactSoft );
	make_soft( 2.0f * contactHertz, d->contactDampingRatio, sc->h, sc->staticSoft );
	make_soft( 0.0f, 0.0f, sc->h, sc->jointSoft );
	sc->restitutionThreshold = d->restitutionThreshold;
	sc->pushout = d->contactPushout;
	sc->gravity = gv( d->gravity.x, d->gravity.y );
	sc->enableWarmStarting = d->enableWarmStarting ? 1 : 0;

	memset( plan, 0, sizeof( *plan ) );
	for ( int c = 0; c <= B2G_COLORS; ++c )
		plan->colorStart[c] = d->colorStart[c];
	for ( int c = 0; c < B2G_OVERFLOW; ++c )
		if ( d->colorStart[c + 1] > d->colorStart[c] )
			plan->active[plan->activeCount++] = c;
	plan->awakeCount = d->bodyCount;

	memset( w, 0, sizeof( *w ) );
	w->state = d->states;
	w->mass = (void*)d->massData;
	w->force = (void*)d->forces;
	w->extent = (void*)d->damping;
	w->awake = (int*)d->bodies;
	w->cBodies = (int*)d->contactBodies;
	w->cMix = (float*)d->contactMix;
	w->manifold = (b2gManifold*)d->manifolds;
	w->solveList = nullptr;
	w->stream = d->stream;
	return 0;
}

/* Points the B2G_ROW_FLOAT4 constraint-row arrays into one block of rows * 144 bytes. */
extern "C" void b2gd_contact_rows( b2gDevWorld* w, void* base, int rows )
{
	char* p = (char*)base;
	size_t n = 16u * (size_t)rows;
	w->kIdx = p;
	w->kNF = p + n;
	w->kMass = p + 2 * n;
	w->kAnchor[0] = p + 3 * n;
	w->kAnchor[1] = p + 4 * n;
	w->kCoef[0] = p + 5 * n;
	w->kCoef[1] = p + 6 * n;
	w->kImp[0] = p + 7 * n;
	w->kImp[1] = p + 8 * n;
	w->solveCap = rows;
}

extern "C" int b2SolveContacts( const b2ContactSolveDesc* desc )
{
	b2gDevWorld w;
	b2gSolvePlan plan;
	b2gStepConst sc;
	if ( b2gd_contact_desc( desc, &w, &plan, &sc ) != 0 )
		return -1;
	cudaStream_t s = (cudaStream_t)desc->stream;
	void* rows = nullptr;
	int n = desc->contactCount > 0 ? desc->contactCount : 1;
	cudaError_t e = cudaMallocAsync( &rows, 16u * B2G_ROW_FLOAT4 * (size_t)n, s );
	if ( e != cudaSuccess )
		return (int)e;
	b2gd_contact_rows( &w, rows, n );
	b2gd_contact_solver( &w, &plan, &sc );
	e = cudaGetLastError();
	cudaError_t f = cudaFreeAsync( rows, s );
	if ( e != cudaSuccess )
		return (int)e;
	return (int)f;
}
