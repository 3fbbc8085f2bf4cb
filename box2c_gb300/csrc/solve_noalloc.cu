/*
 * solve_noalloc.cu -- b2SolveContactsNoAlloc: b2SolveContacts with its constraint rows
 * in a fixed device array compiled into the library, so a call allocates nothing.
 *
 * Who needs it: a host that reserves the device's memory up front (a simulation server
 * or engine that hands its whole budget to its own pool at start-up) has nothing left
 * for a per-call allocation, and a fixed-rate step loop cannot accept an allocation call
 * that may block on other work or fail under memory pressure halfway through a run.
 * Both pass their own buffers and want the solver to take no memory of its own.
 *
 * The rows: B2G_ROW_FLOAT4 float4 arrays of `contactCount` entries carved from one block, the same
 * layout b2SolveContacts uses (b2gd_contact_rows).  k_prepare writes every field of
 * every row before any later kernel reads it, so nothing in the array has to start at
 * zero and nothing is cleared between calls.
 *
 * One array per device: calls that overlap on one device (two host threads, or two
 * streams whose calls are not ordered) write the same rows and race.  The caller orders
 * them.
 */
#include "b2g_device.h"

#include "box2d/gpu.h"

#include <cuda_runtime.h>

#include <mutex>

extern "C" int b2gd_contact_solver( b2gDevWorld* w, const b2gSolvePlan* plan, const b2gStepConst* sc );
extern "C" int b2gd_contact_desc( const b2ContactSolveDesc* d, b2gDevWorld* w, b2gSolvePlan* plan, b2gStepConst* sc );
extern "C" void b2gd_contact_rows( b2gDevWorld* w, void* base, int rows );

/* 144 bytes per contact row: B2G_ROW_FLOAT4 float4 */
static __device__ __align__( 256 ) float4 g_contactRows[B2G_ROW_FLOAT4 * B2_SOLVE_NOALLOC_MAX_CONTACTS];

enum
{
	MAX_DEVICES = 64
};

static std::mutex s_setupLock;
static void* s_rows[MAX_DEVICES];

/* Looks up the array's device address once per device, with that device current.  The
 * lookup may load the library's device code on that device, so the first call on each
 * device belongs before any stream capture starts. */
static int rows_on_current_device( void** out )
{
	int dev = -1;
	cudaError_t e = cudaGetDevice( &dev );
	if ( e != cudaSuccess )
		return (int)e;
	if ( dev < 0 || dev >= MAX_DEVICES )
		return -1;
	std::lock_guard<std::mutex> guard( s_setupLock );
	if ( s_rows[dev] == nullptr )
	{
		void* p = nullptr;
		e = cudaGetSymbolAddress( &p, g_contactRows );
		if ( e != cudaSuccess )
			return (int)e;
		s_rows[dev] = p;
	}
	*out = s_rows[dev];
	return 0;
}

extern "C" int b2SolveContactsNoAlloc( const b2ContactSolveDesc* desc )
{
	b2gDevWorld w;
	b2gSolvePlan plan;
	b2gStepConst sc;
	if ( b2gd_contact_desc( desc, &w, &plan, &sc ) != 0 )
		return -1;
	if ( desc->contactCount > B2_SOLVE_NOALLOC_MAX_CONTACTS )
		return B2_SOLVE_NOALLOC_TOO_LARGE;
	void* rows = nullptr;
	int rc = rows_on_current_device( &rows );
	if ( rc != 0 )
		return rc;
	int n = desc->contactCount > 0 ? desc->contactCount : 1;
	b2gd_contact_rows( &w, rows, n );
	b2gd_contact_solver( &w, &plan, &sc );
	return (int)cudaGetLastError();
}
