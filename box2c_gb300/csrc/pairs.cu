/*
 * pairs.cu -- the broadphase pair query of one world on the device (reference
 * src/broad_phase.c:278-331 b2FindPairsTask over src/dynamic_tree.c:1120
 * b2DynamicTree_Query).
 *
 * One warp per moved proxy walks the kinematic, static (dynamic proxies only) and
 * dynamic trees level by level: the lanes test a level's nodes at once (fat boxes
 * overlap, category non-zero), overlapping leaves are collected and the children of
 * overlapping inner nodes form the next level.  The host query walks depth first with a
 * stack (child1 pushed before child2, so child2's subtree comes first); that order is
 * the order of the leaves' root paths with child2 = 0 and child1 = 1, so every node
 * carries its path as a left-aligned 64-bit key and the warp ranks its leaves by key.
 * The candidate leaves go straight into mapped host memory, where the host pair logic
 * (moved-pair rule, pair set, filters, joints) consumes them in the same order as it
 * would its own query's callbacks; contact creation stays on the host.  The trees are
 * copied up as they are (the host keeps them, b2gTreeNode layout) before each query.
 * A proxy with more candidates than slots, a wider level than the frontier or a deeper
 * tree than the key is left to the host query, which gives the same candidates.
 */
#include "b2g_device.h"

#include <cuda_runtime.h>

#include <stdlib.h>
#include <string.h>

#define QUERY_WARPS 4
#define FRONTIER_CAP 64
#define KEY_DEPTH 62

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

/* One warp's working set: two frontier levels and the leaves of the current tree. */
struct WarpWalk
{
	int node[2][FRONTIER_CAP];
	unsigned long long path[2][FRONTIER_CAP];
	unsigned long long leafPath[B2G_QUERY_SLOTS];
	int2 leaf[B2G_QUERY_SLOTS];
};

/* Appends the overlapping leaves of one tree, in host query order, to out[*found..].
 * Warp-uniform; false when the proxy has to be left to the host query. */
__device__ bool walk_tree( WarpWalk& s, const b2gTreeNode* nodes, int root, int type, b2gBox box, int* found, int2* out )
{
	const unsigned full = 0xFFFFFFFFu;
	const int lane = threadIdx.x & 31;
	const unsigned below = ( 1u << lane ) - 1u;
	int cur = 0, size = 0, leaves = 0;
	if ( root != B2G_NULL )
	{
		if ( lane == 0 )
		{
			s.node[0][0] = root;
			s.path[0][0] = 0ull;
		}
		size = 1;
	}
	__syncwarp();
	for ( int depth = 0; size > 0; ++depth )
	{
		if ( depth >= KEY_DEPTH )
			return false;
		int next = 0;
		for ( int base = 0; base < size; base += 32 )
		{
			int i = base + lane;
			bool isLeaf = false, isInner = false;
			int id = B2G_NULL, child1 = B2G_NULL, child2 = B2G_NULL, shape = 0;
			unsigned long long path = 0ull;
			if ( i < size )
			{
				id = s.node[cur][i];
				path = s.path[cur][i];
				if ( id != B2G_NULL )
				{
					const b2gTreeNode* nd = nodes + id;
					if ( gbox_overlaps( nd->box, box ) && nd->category != 0u )
					{
						if ( nd->height == 0 )
						{
							isLeaf = true;
							shape = nd->userData;
						}
						else
						{
							isInner = true;
							child1 = nd->child1;
							child2 = nd->child2;
						}
					}
				}
			}
			unsigned lm = __ballot_sync( full, isLeaf );
			unsigned im = __ballot_sync( full, isInner );
			int lpos = leaves + __popc( lm & below );
			int ipos = next + 2 * __popc( im & below );
			if ( isLeaf && lpos < B2G_QUERY_SLOTS )
			{
				s.leafPath[lpos] = path;
				s.leaf[lpos] = make_int2( ( id << 2 ) | type, shape );
			}
			if ( isInner && ipos + 1 < FRONTIER_CAP )
			{
				/* child2's subtree comes first in the host walk */
				s.node[cur ^ 1][ipos] = child2;
				s.path[cur ^ 1][ipos] = path;
				s.node[cur ^ 1][ipos + 1] = child1;
				s.path[cur ^ 1][ipos + 1] = path | ( 1ull << ( KEY_DEPTH - depth ) );
			}
			leaves += __popc( lm );
			next += 2 * __popc( im );
		}
		if ( next > FRONTIER_CAP || *found + leaves > B2G_QUERY_SLOTS )
			return false;
		__syncwarp();
		cur ^= 1;
		size = next;
	}
	if ( lane < leaves )
	{
		unsigned long long mine = s.leafPath[lane];
		int rank = 0;
		for ( int j = 0; j < leaves; ++j )
			rank += s.leafPath[j] < mine ? 1 : 0;
		out[*found + rank] = s.leaf[lane];
	}
	*found += leaves;
	__syncwarp();
	return true;
}

__global__ void __launch_bounds__( 32 * QUERY_WARPS ) k_pair_query( const b2gTreeNode* staticNodes, const b2gTreeNode* kinematicNodes,
																 const b2gTreeNode* dynamicNodes, int3 root, const int* keys, int n,
																 int2* cand, int* counts )
{
	__shared__ WarpWalk s_walk[QUERY_WARPS];
	const int w = blockIdx.x * QUERY_WARPS + ( threadIdx.x >> 5 );
	if ( w >= n )
		return;
	WarpWalk& s = s_walk[threadIdx.x >> 5];
	const int lane = threadIdx.x & 31;
	int key = keys[w];
	if ( key == B2G_NULL )
	{
		if ( lane == 0 )
			counts[w] = 0;
		return;
	}
	int type = key & 3;
	int proxy = key >> 2;
	const b2gTreeNode* base = type == 0 ? staticNodes : type == 1 ? kinematicNodes : dynamicNodes;
	b2gBox fat = base[proxy].box;
	int2* out = cand + (size_t)B2G_QUERY_SLOTS * w;
	int found = 0;
	bool whole = true;
	if ( type == 2 )
	{
		whole = walk_tree( s, kinematicNodes, root.y, 1, fat, &found, out );
		whole = whole && walk_tree( s, staticNodes, root.x, 0, fat, &found, out );
	}
	whole = whole && walk_tree( s, dynamicNodes, root.z, 2, fat, &found, out );
	if ( lane == 0 )
		counts[w] = whole ? found : -1;
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
		q = (b2gPairQuery*)b2g_calloc( 1, sizeof( b2gPairQuery ) );
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
		w->h2dBytes += (long long)bytes;
	}
	memcpy( q->hKeys, keys, sizeof( int ) * (size_t)count );
	/* moved-proxy keys are read by the device and counts and candidates written to the
	 * host through mapped memory */
	w->h2dBytes += (long long)( sizeof( int ) * (size_t)count );
	int3 r = make_int3( root[0], root[1], root[2] );
	k_pair_query<<<( count + QUERY_WARPS - 1 ) / QUERY_WARPS, 32 * QUERY_WARPS, 0, s>>>(
		q->nodes[0], q->nodes[1], q->nodes[2], r, q->dKeys, count, (int2*)q->dCand, q->dCount );
	cudaError_t e = cudaGetLastError();
	if ( e == cudaSuccess )
		e = cudaStreamSynchronize( s );
	*cand = q->hCand;
	*counts = q->hCount;
	if ( e == cudaSuccess )
	{
		long long n = 0;
		for ( int i = 0; i < count; ++i )
			n += q->hCount[i] > 0 ? q->hCount[i] : 0;
		w->d2hBytes += (long long)sizeof( int ) * ( (long long)count + 2 * n );
	}
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
	b2g_free( q );
}
