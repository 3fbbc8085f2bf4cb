/*
 * b2g_packs.h -- how the batched solver lays out its worlds: the shared-memory image of
 * one world (body states, then its rows when they fit) and the packs of similar-sized
 * worlds that one CTA solves side by side.  Host code (and the two size functions for the
 * device), shared by batch.cu and the host test of the packing.
 */
#pragma once

#include "b2g_device.h"

#include <stddef.h>
#include <string.h>

#ifdef __CUDACC__
#define B2G_PACK_HD __host__ __device__
#else
#define B2G_PACK_HD
#endif

/* Shared-memory image of one world on its solver group: body states (two float4) by
 * body id; after them, for a world that fits, its constraint rows by solve-list
 * position (nine float4 each).  Velocity terms are recomputed every substep from the
 * body's mass, force and extent rather than held, which keeps the image small. */
B2G_PACK_HD inline int body_float4s( int bodies ) { return 2 * bodies; }
B2G_PACK_HD inline size_t world_smem_bytes( int bodies, int rows )
{
	return 16u * (size_t)body_float4s( bodies ) + 144u * (size_t)rows;
}

/* A pack: worlds of similar size solved side by side by one CTA, each by a group of
 * `group` threads with 1 / (T / group) of the CTA's shared memory. */
#define PACK_WORLDS 16
#define PACK_INTS ( 1 + PACK_WORLDS )

/* Builds the packs of items [first, first + n) for CTAs of T threads with smem bytes of
 * shared memory into order ([0] packs, then PACK_INTS ints per pack: group size, item
 * indices or -1; 1 + 2 * PACK_INTS * n ints, the second half scratch), using scratch
 * (5 * n ints).  smem holds the largest world's bodies (32 bytes each).  Each world gets the smallest group (32 ..
 * T threads, powers of two) that holds its bodies in the group's share of shared
 * memory and covers its widest colour in two passes when its rows fit in that share too
 * (they are then kept on chip), in one pass otherwise.  Worlds of one group size are
 * packed largest first; packs go into the queue by their longest world (colours x
 * passes), then alternating from both ends.  Returns the number of packs. */
static inline int b2g_build_packs( b2gBatchItem* items, int first, int n, int T, size_t smem, int* scratch, int* order )
{
	/* per item of the half (local index): */
	int* groupOf = scratch;			/* group size, 0 when not solved */
	int* byGroup = scratch + n;		/* local indices by group size, largest first */
	int* packCost = scratch + 2 * n; /* per pack */
	int* sizeKey = scratch + 3 * n;	/* body count */
	int* cost = scratch + 4 * n;	/* colours x passes */
	int* packs = order + 1;
	int* tmp = order + 1 + PACK_INTS * n;
	int top = 1;
	for ( int i = 0; i < n; ++i )
	{
		b2gBatchItem& it = items[first + i];
		it.rowsOnChip = 0;
		groupOf[i] = 0;
		if ( it.solve == 0 )
			continue;
		/* rows on chip: two passes per colour; rows in global memory: one, so that fewer
		 * such worlds are resident at once and their rows stay in L2 */
		int g = 32;
		bool onChip = false;
		for ( ;; )
		{
			size_t share = ( smem / (size_t)( T / g ) ) / 16u * 16u;
			onChip = world_smem_bytes( it.bodyIdCount, it.colorStart[B2G_COLORS] ) <= share;
			bool bodiesFit = 32u * (size_t)it.bodyIdCount <= share;
			if ( g >= T || ( bodiesFit && ( onChip ? 2 : 1 ) * g >= it.widest ) )
				break;
			g *= 2;
		}
		groupOf[i] = g;
		it.rowsOnChip = onChip ? 1 : 0;
		sizeKey[i] = it.bodyIdCount;
		cost[i] = ( it.activeCount + 1 ) * ( ( it.widest + g - 1 ) / g + 1 );
		top = it.bodyIdCount > top ? it.bodyIdCount : top;
	}
	/* counting sort on (group size, body count): 5 group sizes (32 .. 512) x 64 size buckets */
	const int buckets = 64;
	const int groups = 5;
	int count[groups * buckets + 1];
	memset( count, 0, sizeof( count ) );
	auto key = [&]( int i ) {
		int gk = 0;
		for ( int g = groupOf[i]; g > 32; g >>= 1 )
			gk += 1;
		return gk * buckets + buckets - 1 - (int)( (long long)sizeKey[i] * ( buckets - 1 ) / top );
	};
	for ( int i = 0; i < n; ++i )
		if ( groupOf[i] )
			count[key( i )] += 1;
	for ( int k = 0, s = 0; k <= groups * buckets; ++k )
	{
		int c = count[k];
		count[k] = s;
		s += c;
	}
	int m = count[groups * buckets];
	for ( int i = 0; i < n; ++i )
		if ( groupOf[i] )
			byGroup[count[key( i )]++] = i;
	/* packs of T / g consecutive worlds of one group size */
	int P = 0, costTop = 1;
	for ( int k = 0; k < m; )
	{
		int g = groupOf[byGroup[k]];
		int* p = tmp + PACK_INTS * P;
		p[0] = g;
		int most = 0;
		for ( int j = 0; j < PACK_WORLDS; ++j )
		{
			bool take = j < T / g && k < m && groupOf[byGroup[k]] == g;
			int li = take ? byGroup[k++] : -1;
			p[1 + j] = take ? first + li : -1;
			if ( take )
				most = cost[li] > most ? cost[li] : most;
		}
		packCost[P++] = most;
		costTop = most > costTop ? most : costTop;
	}
	/* queue order: costliest first (counting sort), then alternating from both ends */
	int ccount[buckets + 1];
	memset( ccount, 0, sizeof( ccount ) );
	auto ckey = [&]( int q ) { return buckets - 1 - (int)( (long long)packCost[q] * ( buckets - 1 ) / costTop ); };
	for ( int q = 0; q < P; ++q )
		ccount[ckey( q )] += 1;
	for ( int k = 0, s = 0; k <= buckets; ++k )
	{
		int c = ccount[k];
		ccount[k] = s;
		s += c;
	}
	int* sorted = byGroup; /* reused: pack indices by cost */
	for ( int q = 0; q < P; ++q )
		sorted[ccount[ckey( q )]++] = q;
	for ( int i = 0, lo = 0, hi = P - 1; lo <= hi; ++i )
	{
		int q = ( i & 1 ) == 0 ? sorted[lo++] : sorted[hi--];
		memcpy( packs + PACK_INTS * i, tmp + PACK_INTS * q, sizeof( int ) * PACK_INTS );
	}
	order[0] = P;
	return P;
}
