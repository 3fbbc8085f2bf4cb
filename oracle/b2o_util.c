/*
 * b2o_util.c -- containers of the plain-C oracle (TEST INFRASTRUCTURE).
 *
 * Restates the semantics the step path depends on: swap-remove arrays (reference
 * src/block_array.c), the LIFO id pool (src/id_pool.c:21-45), bit sets (src/bitset.c)
 * and a membership-only hash set (src/table.c).
 */
#include "b2o.h"

#include <string.h>

void oia_push( oIntArray* a, int v )
{
	if ( a->count == a->capacity )
	{
		int cap = a->capacity < 16 ? 16 : 2 * a->capacity;
		a->data = (int*)realloc( a->data, sizeof( int ) * cap );
		a->capacity = cap;
	}
	a->data[a->count++] = v;
}

int oia_remove_swap( oIntArray* a, int index )
{
	int last = a->count - 1;
	if ( index == last )
	{
		a->count -= 1;
		return -1;
	}
	a->data[index] = a->data[last];
	a->count -= 1;
	return last;
}

void oia_free( oIntArray* a )
{
	free( a->data );
	memset( a, 0, sizeof( *a ) );
}

static uint64_t oset_hash( uint64_t k )
{
	k ^= k >> 33;
	k *= 0xff51afd7ed558ccdULL;
	k ^= k >> 33;
	k *= 0xc4ceb9fe1a85ec53ULL;
	k ^= k >> 33;
	return k;
}

static void oset_grow( oSet* s )
{
	int oldCap = s->capacity;
	uint64_t* old = s->keys;
	s->capacity = oldCap == 0 ? 64 : 2 * oldCap;
	s->keys = (uint64_t*)calloc( (size_t)s->capacity, sizeof( uint64_t ) );
	s->count = 0;
	for ( int i = 0; i < oldCap; ++i )
		if ( old[i] != 0 )
			oset_add( s, old[i] );
	free( old );
}

bool oset_add( oSet* s, uint64_t key )
{
	if ( 2 * ( s->count + 1 ) > s->capacity )
		oset_grow( s );
	uint64_t mask = (uint64_t)( s->capacity - 1 );
	uint64_t i = oset_hash( key ) & mask;
	while ( s->keys[i] != 0 )
	{
		if ( s->keys[i] == key )
			return true;
		i = ( i + 1 ) & mask;
	}
	s->keys[i] = key;
	s->count += 1;
	return false;
}

bool oset_contains( const oSet* s, uint64_t key )
{
	if ( s->capacity == 0 )
		return false;
	uint64_t mask = (uint64_t)( s->capacity - 1 );
	uint64_t i = oset_hash( key ) & mask;
	while ( s->keys[i] != 0 )
	{
		if ( s->keys[i] == key )
			return true;
		i = ( i + 1 ) & mask;
	}
	return false;
}

bool oset_remove( oSet* s, uint64_t key )
{
	if ( s->capacity == 0 )
		return false;
	uint64_t mask = (uint64_t)( s->capacity - 1 );
	uint64_t i = oset_hash( key ) & mask;
	while ( s->keys[i] != 0 && s->keys[i] != key )
		i = ( i + 1 ) & mask;
	if ( s->keys[i] == 0 )
		return false;
	/* backward-shift deletion keeps probe chains intact */
	s->keys[i] = 0;
	s->count -= 1;
	uint64_t j = ( i + 1 ) & mask;
	while ( s->keys[j] != 0 )
	{
		uint64_t k = s->keys[j];
		s->keys[j] = 0;
		s->count -= 1;
		oset_add( s, k );
		j = ( j + 1 ) & mask;
	}
	return true;
}

void oset_clear( oSet* s )
{
	if ( s->keys )
		memset( s->keys, 0, sizeof( uint64_t ) * (size_t)s->capacity );
	s->count = 0;
}

void oset_free( oSet* s )
{
	free( s->keys );
	memset( s, 0, sizeof( *s ) );
}

int oid_alloc( oIdPool* p )
{
	if ( p->freeIds.count > 0 )
	{
		p->freeIds.count -= 1;
		return p->freeIds.data[p->freeIds.count];
	}
	return p->next++;
}

void oid_free( oIdPool* p, int id )
{
	oia_push( &p->freeIds, id );
}

int oid_count( const oIdPool* p )
{
	return p->next - p->freeIds.count;
}

bool obits_get( const oBits* b, int i )
{
	int w = i >> 6;
	if ( w >= b->wordCount )
		return false;
	return ( b->words[w] >> ( i & 63 ) ) & 1u;
}

void obits_set( oBits* b, int i )
{
	int w = i >> 6;
	if ( w >= b->wordCount )
	{
		int n = 2 * ( w + 1 );
		b->words = (uint64_t*)realloc( b->words, sizeof( uint64_t ) * n );
		memset( b->words + b->wordCount, 0, sizeof( uint64_t ) * ( n - b->wordCount ) );
		b->wordCount = n;
	}
	b->words[w] |= (uint64_t)1 << ( i & 63 );
}

void obits_clear( oBits* b, int i )
{
	int w = i >> 6;
	if ( w < b->wordCount )
		b->words[w] &= ~( (uint64_t)1 << ( i & 63 ) );
}

void obits_free( oBits* b )
{
	free( b->words );
	memset( b, 0, sizeof( *b ) );
}
