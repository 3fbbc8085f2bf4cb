/*
 * pairs.cu -- the broadphase pair query of one world on the device (reference
 * src/broad_phase.c:278-331 b2FindPairsTask over src/dynamic_tree.c:1120
 * b2DynamicTree_Query).
 *
 * One thread per moved proxy walks the kinematic, static (dynamic proxies only) and
 * dynamic trees from their roots with its own stack, in the host query's order: a node
 * whose fat box overlaps the proxy's fat box and whose category is non-zero is reported
 * if it is a leaf, otherwise child1 then child2 are pushed (so child2 is visited first).
 * The candidate leaves go straight into mapped host memory, where the host pair logic
 * (moved-pair rule, pair set, filters, joints) consumes them in the same order as it
 * would its own query's callbacks; contact creation stays on the host.  The trees are
 * copied up as they are (the host keeps them, b2gTreeNode layout) before each query.
 */
#include "b2g_device.h"

#include <cuda_runtime.h>

#include <stdlib.h>
#include <string.h>

#define QUERY_STACK 64
#define QUERY_THREADS 128

struct b2gPairQuery
{
	b2gTreeNode* nodes[3];
	size_t nodeBytes[3];
	int* hKeys; /* mapped: moved proxy keys */
	int* dKeys;
	int* hCand; /* mapped: B2G_QUERY_SLOTS (key, shape) pairs per moved proxy */
	int* dCand;
	int* hCount; /* mapped: candidates per moved proxy, -1 when the host must query */
	int* dCount;
	int cap;
};

/* One tree walk; false when the stack would overflow (the host then queries). */
__device__ bool walk_tree( const b2gTreeNode* nodes, int root, int type, b2gBox box, int* found, int2* out )
{
	int stack[QUERY_STACK];
	int n = 0;
	stack[n++] = root;
	while ( n > 0 )
	{
		int id = stack[--n];
		if ( id == B2G_NULL )
			continue;
		const b2gTreeNode* node = nodes + id;
		if ( gbox_overlaps( node->box, box ) && node->category != 0u )
		{
			if ( node->height == 0 )
			{
				if ( *found < B2G_QUERY_SLOTS )
					out[*found] = make_int2( ( id << 2 ) | type, node->userData );
				*found += 1;
			}
			else
			{
				if ( n >= QUERY_STACK - 1 )
					return false;
				stack[n++] = node->child1;
				stack[n++] = node->child2;
			}
		}
	}
	return true;
}

__global__ void __launch_bounds__( QUERY_THREADS ) k_pair_query( const b2gTreeNode* staticNodes, const b2gTreeNode* kinematicNodes,
															   const b2gTreeNode* dynamicNodes, int3 root, const int* keys, int n,
															   int2* cand, int* counts )
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if ( i >= n )
		return;
	int key = keys[i];
	if ( key == B2G_NULL )
	{
		counts[i] = 0;
		return;
	}
	int type = key & 3;
	int proxy = key >> 2;
	const b2gTreeNode* base = type == 0 ? staticNodes : type == 1 ? kinematicNodes : dynamicNodes;
	b2gBox fat = base[proxy].box;
	int2* out = cand + (size_t)B2G_QUERY_SLOTS * i;
	int found = 0;
	bool whole = true;
	if ( type == 2 )
	{
		whole = walk_tree( kinematicNodes, root.y, 1, fat, &found, out );
		whole = whole && walk_tree( staticNodes, root.x, 0, fat, &found, out );
	}
	whole = whole && walk_tree( dynamicNodes, root.z, 2, fat, &found, out );
	counts[i] = whole && found <= B2G_QUERY_SLOTS ? found : -1;
}

static int mapped( void** h, void** d, size_t bytes )
{
	if ( cudaHostAlloc( h, bytes, cudaHostAllocMapped ) != cudaSuccess )
		return (int)cudaErrorMemoryAllocation;
	return (int)cudaHostGetDevicePointer( d, *h, 0 );
}

static void release_mapped( b2gPairQuery* q )
{
	if ( q->hKeys )
		cudaFreeHost( q->hKeys );
	if ( q->hCand )
		cudaFreeHost( q->hCand );
	if ( q->hCount )
		cudaFreeHost( q->hCount );
	q->hKeys = q->dKeys = q->hCand = q->dCand = q->hCount = q->dCount = nullptr;
	q->cap = 0;
}

extern "C" int b2gd_pair_query( b2gDevWorld* w, b2gPairQuery** query, const b2gTreeNode* const nodes[3], const int capacity[3],
								const int root[3], const int* keys, int count, const int** cand, const int** counts )
{
	cudaStream_t s = (cudaStream_t)w->stream;
	b2gPairQuery* q = *query;
	if ( q == nullptr )
	{
		q = (b2gPairQuery*)calloc( 1, sizeof( b2gPairQuery ) );
		if ( q == nullptr )
			return (int)cudaErrorMemoryAllocation;
		*query = q;
	}
	if ( count > q->cap )
	{
		cudaStreamSynchronize( s );
		release_mapped( q );
		int cap = count > 256 ? count : 256;
		int e = mapped( (void**)&q->hKeys, (void**)&q->dKeys, sizeof( int ) * (size_t)cap );
		if ( e == 0 )
			e = mapped( (void**)&q->hCand, (void**)&q->dCand, sizeof( int ) * 2u * B2G_QUERY_SLOTS * (size_t)cap );
		if ( e == 0 )
			e = mapped( (void**)&q->hCount, (void**)&q->dCount, sizeof( int ) * (size_t)cap );
		if ( e )
		{
			release_mapped( q );
			return e;
		}
		q->cap = cap;
	}
	for ( int t = 0; t < 3; ++t )
	{
		size_t bytes = sizeof( b2gTreeNode ) * (size_t)capacity[t];
		if ( bytes > q->nodeBytes[t] )
		{
			if ( q->nodes[t] )
				cudaFreeAsync( q->nodes[t], s );
			q->nodes[t] = nullptr;
			q->nodeBytes[t] = 0;
			if ( cudaMallocAsync( (void**)&q->nodes[t], 2 * bytes, s ) != cudaSuccess )
				return (int)cudaErrorMemoryAllocation;
			q->nodeBytes[t] = 2 * bytes;
		}
		if ( bytes > 0 )
			cudaMemcpyAsync( q->nodes[t], nodes[t], bytes, cudaMemcpyHostToDevice, s );
	}
	memcpy( q->hKeys, keys, sizeof( int ) * (size_t)count );
	int3 r = make_int3( root[0], root[1], root[2] );
	k_pair_query<<<( count + QUERY_THREADS - 1 ) / QUERY_THREADS, QUERY_THREADS, 0, s>>>(
		q->nodes[0], q->nodes[1], q->nodes[2], r, q->dKeys, count, (int2*)q->dCand, q->dCount );
	cudaError_t e = cudaGetLastError();
	if ( e == cudaSuccess )
		e = cudaStreamSynchronize( s );
	*cand = q->hCand;
	*counts = q->hCount;
	return (int)e;
}

extern "C" void b2gd_pair_query_free( b2gPairQuery* q )
{
	if ( q == nullptr )
		return;
	for ( int t = 0; t < 3; ++t )
		if ( q->nodes[t] )
			cudaFree( q->nodes[t] );
	release_mapped( q );
	free( q );
}
