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
 * Before a leaf is kept, the warp applies the pair rules that reject nearly every
 * candidate (src/broad_phase.c:170-205): the proxy itself, a moved non-static proxy with
 * a smaller key (its own query reports the pair), and a shape pair that already has a
 * contact (the host's pair set, copied up as it is whenever it changed: same table, same
 * hash, same probing).  The remaining leaves go into mapped host memory in the order of
 * the host query, where the host applies the rest of the pair logic (filters, sensors,
 * joints) exactly as it would in its own query's callbacks; contact creation stays on
 * the host.  The trees are
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
	unsigned long long* pairs; /* copy of the host pair set's table */
	int pairCap;
	unsigned pairVersion; /* version of the host pair set the copy holds */
	bool pairsValid;
	int* moved; /* per proxy key: the query stamp when the proxy moved */
	int movedCap;
	int stamp;
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

/* The host pair set's hash (util.c gset_hash) and linear probing; 0 marks a free slot. */
__device__ __forceinline__ unsigned long long pair_hash( unsigned long long k )
{
	k ^= k >> 33;
	k *= 0xff51afd7ed558ccdULL;
	k ^= k >> 33;
	k *= 0xc4ceb9fe1a85ec53ULL;
	k ^= k >> 33;
	return k;
}

__device__ bool pair_exists( const unsigned long long* table, int cap, unsigned long long key )
{
	if ( cap == 0 )
		return false;
	unsigned long long mask = (unsigned long long)( cap - 1 );
	unsigned long long i = pair_hash( key ) & mask;
	for ( int probe = 0; probe < cap; ++probe )
	{
		unsigned long long k = table[i];
		if ( k == 0ull )
			return false;
		if ( k == key )
			return true;
		i = ( i + 1 ) & mask;
	}
	return false;
}

/* What the device knows of the pair rules for one query. */
struct PairFilter
{
	const unsigned long long* pairs;
	int pairCap;
	const int* moved;
	int stamp;
	int queryKey;
	int queryShape;
};

/* True when the host's pair rules would reject the candidate for one of the reasons the
 * device can see (reference src/broad_phase.c:170-205). */
__device__ __forceinline__ bool rejected( const PairFilter& f, int proxyKey, int shape )
{
	if ( proxyKey == f.queryKey )
		return true;
	if ( ( proxyKey & 3 ) != 0 && f.moved[proxyKey] == f.stamp && proxyKey < f.queryKey )
		return true;
	unsigned long long a = (unsigned long long)(unsigned)shape, b = (unsigned long long)(unsigned)f.queryShape;
	unsigned long long key = a < b ? ( a << 32 | b ) : ( b << 32 | a );
	return pair_exists( f.pairs, f.pairCap, key );
}

/* Appends the overlapping leaves of one tree that pass the device's pair rules, in host
 * query order, to out[*found..].  Warp-uniform; false when the proxy has to be left to
 * the host query (the slot limit counts every overlapping leaf). */
__device__ bool walk_tree( WarpWalk& s, const b2gTreeNode* nodes, int root, int type, b2gBox box, int* found, int2* out,
						   int* seen, const PairFilter& filter )
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
		if ( next > FRONTIER_CAP || *seen + leaves > B2G_QUERY_SLOTS )
			return false;
		__syncwarp();
		cur ^= 1;
		size = next;
	}
	/* rank the leaves by root path (host order), then keep the ones the rules pass,
	 * in that order */
	int rank = 0;
	bool keep = false;
	if ( lane < leaves )
	{
		unsigned long long mine = s.leafPath[lane];
		for ( int j = 0; j < leaves; ++j )
			rank += s.leafPath[j] < mine ? 1 : 0;
		keep = rejected( filter, s.leaf[lane].x, s.leaf[lane].y ) == false;
	}
	unsigned km = __ballot_sync( full, keep );
	int pos = 0;
	for ( int j = 0; j < leaves; ++j )
	{
		bool other = ( ( km >> j ) & 1u ) != 0;
		int otherRank = __shfl_sync( full, rank, j );
		pos += ( other && otherRank < rank ) ? 1 : 0;
	}
	if ( keep )
		out[*found + pos] = s.leaf[lane];
	*found += __popc( km );
	*seen += leaves;
	__syncwarp();
	return true;
}

/* Stamps the moved proxies of this query (the moved-pair rule reads the stamps). */
__global__ void k_mark_moved( const int* keys, int n, int* moved, int stamp )
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if ( i < n && keys[i] != B2G_NULL )
		moved[keys[i]] = stamp;
}

__global__ void __launch_bounds__( 32 * QUERY_WARPS ) k_pair_query( const b2gTreeNode* staticNodes, const b2gTreeNode* kinematicNodes,
																 const b2gTreeNode* dynamicNodes, int3 root, const int* keys, int n,
																 int2* cand, int* counts, const unsigned long long* pairs, int pairCap,
																 const int* moved, int stamp )
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
	PairFilter filter = { pairs, pairCap, moved, stamp, key, base[proxy].userData };
	int found = 0, seen = 0;
	bool whole = true;
	if ( type == 2 )
	{
		whole = walk_tree( s, kinematicNodes, root.y, 1, fat, &found, out, &seen, filter );
		whole = whole && walk_tree( s, staticNodes, root.x, 0, fat, &found, out, &seen, filter );
	}
	whole = whole && walk_tree( s, dynamicNodes, root.z, 2, fat, &found, out, &seen, filter );
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
								const int root[3], const int* keys, int count, const unsigned long long* pairTable, int pairCap,
								unsigned pairVersion, const int** cand, const int** counts )
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
	/* the host pair set's table, copied when it changed since the last query */
	if ( q->pairsValid == false || q->pairVersion != pairVersion || q->pairCap != pairCap )
	{
		if ( pairCap > q->pairCap || q->pairs == nullptr )
		{
			if ( q->pairs )
				cudaFreeAsync( q->pairs, s );
			q->pairs = nullptr;
			q->pairsValid = false;
			if ( pairCap > 0 && cudaMallocAsync( (void**)&q->pairs, sizeof( unsigned long long ) * (size_t)pairCap, s ) != cudaSuccess )
				return (int)cudaErrorMemoryAllocation;
		}
		if ( pairCap > 0 )
		{
			cudaMemcpyAsync( q->pairs, pairTable, sizeof( unsigned long long ) * (size_t)pairCap, cudaMemcpyHostToDevice, s );
			w->h2dBytes += (long long)( sizeof( unsigned long long ) * (size_t)pairCap );
		}
		q->pairCap = pairCap;
		q->pairVersion = pairVersion;
		q->pairsValid = true;
	}
	/* stamps of moved proxies, indexed by proxy key */
	int maxCap = capacity[0] > capacity[1] ? capacity[0] : capacity[1];
	maxCap = maxCap > capacity[2] ? maxCap : capacity[2];
	if ( 4 * maxCap > q->movedCap )
	{
		if ( q->moved )
			cudaFreeAsync( q->moved, s );
		int cap = 8 * maxCap;
		if ( cudaMallocAsync( (void**)&q->moved, sizeof( int ) * (size_t)cap, s ) != cudaSuccess )
		{
			q->moved = nullptr;
			q->movedCap = 0;
			return (int)cudaErrorMemoryAllocation;
		}
		cudaMemsetAsync( q->moved, 0, sizeof( int ) * (size_t)cap, s );
		q->movedCap = cap;
	}
	q->stamp = q->stamp == 0x7FFFFFFF ? 1 : q->stamp + 1;
	memcpy( q->hKeys, keys, sizeof( int ) * (size_t)count );
	/* moved-proxy keys are read by the device and counts and candidates written to the
	 * host through mapped memory */
	w->h2dBytes += (long long)( sizeof( int ) * (size_t)count );
	int3 r = make_int3( root[0], root[1], root[2] );
	k_mark_moved<<<( count + 255 ) / 256, 256, 0, s>>>( q->dKeys, count, q->moved, q->stamp );
	k_pair_query<<<( count + QUERY_WARPS - 1 ) / QUERY_WARPS, 32 * QUERY_WARPS, 0, s>>>(
		q->nodes[0], q->nodes[1], q->nodes[2], r, q->dKeys, count, (int2*)q->dCand, q->dCount, q->pairs, q->pairCap, q->moved,
		q->stamp );
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
	if ( q->pairs )
		cudaFree( q->pairs );
	if ( q->moved )
		cudaFree( q->moved );
	release_mapped( q );
	b2g_free( q );
}
