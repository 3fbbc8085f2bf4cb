/*
 * packs_check.cpp -- host check of the batched solver's packing (b2g_packs.h) on seeded
 * random batches: every solving world lands in exactly one pack and no other world does;
 * a pack's group size is a power of two from 32 to T and holds at most T / group worlds;
 * each world's group holds its bodies in its share of shared memory, is the smallest
 * that does so while covering the widest colour in two passes (rows on chip) or one
 * (rows in global memory), and rows are marked on chip exactly when they fit the share;
 * the first pack in the queue is the costliest.  Prints "ok" or the first failure.
 */
#include "b2g_packs.h"

#include <stdio.h>
#include <stdlib.h>
#include <vector>

static unsigned long long s_state = 12345;
static int rnd( int lo, int hi )
{
	s_state = s_state * 6364136223846793005ull + 1442695040888963407ull;
	return lo + (int)( ( s_state >> 33 ) % (unsigned long long)( hi - lo + 1 ) );
}

static size_t share_of( size_t smem, int T, int g ) { return ( smem / (size_t)( T / g ) ) / 16u * 16u; }

static bool fits( const b2gBatchItem& it, size_t smem, int T, int g, bool* onChip )
{
	size_t share = share_of( smem, T, g );
	*onChip = world_smem_bytes( it.bodyIdCount, it.colorStart[B2G_COLORS] ) <= share;
	bool bodies = 32u * (size_t)it.bodyIdCount <= share;
	return bodies && ( *onChip ? 2 : 1 ) * g >= it.widest;
}

static int fail( const char* what, int T, int n )
{
	printf( "failed: %s (T %d, n %d)\n", what, T, n );
	return 1;
}

int main()
{
	const int Ts[4] = { 64, 128, 256, 512 };
	for ( int trial = 0; trial < 40; ++trial )
	{
		int n = rnd( 1, 3000 );
		int first = rnd( 0, 50 );
		std::vector<b2gBatchItem> items( (size_t)( first + n ) );
		int top = 0;
		for ( int i = first; i < first + n; ++i )
		{
			b2gBatchItem& it = items[i];
			memset( &it, 0, sizeof( it ) );
			it.solve = rnd( 0, 9 ) != 0;
			int b = rnd( 4, trial % 5 == 0 ? 118 : 40 );
			it.bodyIdCount = b * ( b + 1 ) / 2 + 1;
			int rows = 3 * it.bodyIdCount;
			it.colorStart[B2G_COLORS] = rows;
			it.activeCount = rnd( 1, 11 );
			it.widest = rnd( 1, rows / it.activeCount + 1 );
			if ( it.solve )
				top = it.bodyIdCount > top ? it.bodyIdCount : top;
		}
		for ( int t = 0; t < 4; ++t )
		{
			const int T = Ts[t];
			size_t target = (size_t)rnd( 12, 222 ) * 1024u;
			size_t smem = 16u * (size_t)body_float4s( ( top + 255 ) / 256 * 256 );
			smem = smem > target ? smem : target;
			std::vector<int> scratch( 5u * (size_t)( n + 1 ) ), order( 1u + 2u * PACK_INTS * (size_t)( n + 1 ) );
			int P = b2g_build_packs( items.data(), first, n, T, smem, scratch.data(), order.data() );
			if ( P != order[0] )
				return fail( "pack count", T, n );
			std::vector<int> seen( items.size(), 0 );
			int lastCost = -1;
			for ( int q = 0; q < P; ++q )
			{
				const int* p = order.data() + 1 + PACK_INTS * q;
				int g = p[0];
				if ( g < 32 || g > T || ( g & ( g - 1 ) ) != 0 )
					return fail( "group size", T, n );
				int worlds = 0, cost = 0;
				for ( int j = 0; j < PACK_WORLDS; ++j )
				{
					int w = p[1 + j];
					if ( w < 0 )
						continue;
					if ( j >= T / g )
						return fail( "more worlds than groups in a pack", T, n );
					if ( w < first || w >= first + n || items[w].solve == 0 )
						return fail( "a world outside the batch or not solving", T, n );
					seen[w] += 1;
					worlds += 1;
					bool onChip;
					if ( fits( items[w], smem, T, g, &onChip ) == false && g < T )
						return fail( "group too small", T, n );
					if ( g > 32 && fits( items[w], smem, T, g / 2, &onChip ) )
						return fail( "group not the smallest", T, n );
					fits( items[w], smem, T, g, &onChip );
					if ( items[w].rowsOnChip != ( onChip ? 1 : 0 ) )
						return fail( "rows on chip", T, n );
					if ( 32u * (size_t)items[w].bodyIdCount > share_of( smem, T, g ) )
						return fail( "bodies do not fit the share", T, n );
					int c = ( items[w].activeCount + 1 ) * ( ( items[w].widest + g - 1 ) / g + 1 );
					cost = c > cost ? c : cost;
				}
				if ( worlds == 0 )
					return fail( "an empty pack", T, n );
				if ( q == 0 )
					lastCost = cost;
			}
			for ( int w = first; w < first + n; ++w )
				if ( seen[w] != ( items[w].solve ? 1 : 0 ) )
					return fail( "every solving world in exactly one pack", T, n );
			/* the queue starts with a costliest pack (cost buckets of 1/64 of the top) */
			int most = 0;
			for ( int q = 0; q < P; ++q )
			{
				const int* p = order.data() + 1 + PACK_INTS * q;
				for ( int j = 0; j < PACK_WORLDS; ++j )
				{
					int w = p[1 + j];
					if ( w < 0 )
						continue;
					int c = ( items[w].activeCount + 1 ) * ( ( items[w].widest + p[0] - 1 ) / p[0] + 1 );
					most = c > most ? c : most;
				}
			}
			if ( P > 0 && (long long)lastCost * 64 < (long long)most * 63 )
				return fail( "the queue starts with a costliest pack", T, n );
		}
	}
	printf( "ok\n" );
	return 0;
}
