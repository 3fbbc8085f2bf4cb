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

/* The array's address in each device's current context, with the id of that context:
 * a context made after cudaDeviceReset loads the library's device code anew, so its
 * address is looked up again. */
typedef struct RowsAddress
{
	void* rows;
	unsigned long long context;
} RowsAddress;

static std::mutex s_setupLock;
static RowsAddress s_rows[MAX_DEVICES];

typedef int ( *CtxGetCurrentFn )( void** ctx );
typedef int ( *CtxGetIdFn )( void* ctx, unsigned long long* id );

/* Id of the current context through the driver's entry points (no link to the driver
 * library); 0 when the driver does not provide them, and then the address is kept per
 * device ordinal only. */
static unsigned long long current_context_id( void )
{
	static CtxGetCurrentFn getCurrent;
	static CtxGetIdFn getId;
	static bool looked;
	if ( looked == false )
	{
		cudaDriverEntryPointQueryResult q;
		void* f = nullptr;
		if ( cudaGetDriverEntryPointByVersion( "cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q ) == cudaSuccess &&
			 q == cudaDriverEntryPointSuccess )
			getCurrent = (CtxGetCurrentFn)f;
		f = nullptr;
		if ( cudaGetDriverEntryPointByVersion( "cuCtxGetId", &f, 12000, cudaEnableDefault, &q ) == cudaSuccess &&
			 q == cudaDriverEntryPointSuccess )
			getId = (CtxGetIdFn)f;
		looked = true;
	}
	void* ctx = nullptr;
	unsigned long long id = 0;
	if ( getCurrent == nullptr || getId == nullptr || getCurrent( &ctx ) != 0 || ctx == nullptr || getId( ctx, &id ) != 0 )
		return 0;
	return id;
}

/* Looks up the array's device address once per device (and again after the device's
 * context was replaced), with that device current.  The lookup may load the library's
 * device code on that device, so the first call on each device belongs before any
 * stream capture starts. */
static int rows_on_current_device( void** out )
{
	int dev = -1;
	cudaError_t e = cudaGetDevice( &dev );
	if ( e != cudaSuccess )
		return (int)e;
	if ( dev < 0 || dev >= MAX_DEVICES )
		return B2_SOLVE_NOALLOC_DEVICE_LIMIT;
	std::lock_guard<std::mutex> guard( s_setupLock );
	RowsAddress* a = s_rows + dev;
	if ( a->rows == nullptr || a->context != current_context_id() )
	{
		void* p = nullptr;
		e = cudaGetSymbolAddress( &p, g_contactRows );
		if ( e != cudaSuccess )
			return (int)e;
		a->rows = p;
		/* the lookup has made the device's context current: its id keys the address */
		a->context = current_context_id();
	}
	*out = a->rows;
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
