/*
 * util.c -- host containers of the step driver.
 *
 * Restates the semantics the step path depends on: swap-remove arrays (reference
 * src/block_array.c), the LIFO id pool (src/id_pool.c:21-45), bit sets (src/bitset.c)
 * and a membership-only hash set (src/table.c).
 */
#include "host.h"

#include <string.h>

void gia_push( gIntArray* a, int v )
{
	if ( a->count == a->capacity )
	{
		int cap = a->capacity < 16 ? 16 : 2 * a->capacity;
		a->data = (int*)realloc( a->data, sizeof( int ) * cap );
		a->capacity = cap;
	}
	a->data[a->count++] = v;
}

int gia_remove_swap( gIntArray* a, int index )
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

void gia_free( gIntArray* a )
{
	free( a->data );
	memset( a, 0, sizeof( *a ) );
}

static uint64_t gset_hash( uint64_t k )
{
	k ^= k >> 33;
	k *= 0xff51afd7ed558ccdULL;
	k ^= k >> 33;
	k *= 0xc4ceb9fe1a85ec53ULL;
	k ^= k >> 33;
	return k;
}

static void gset_grow( gSet* s )
{
	int oldCap = s->capacity;
	uint64_t* old = s->keys;
	s->capacity = oldCap == 0 ? 64 : 2 * oldCap;
	s->keys = (uint64_t*)calloc( (size_t)s->capacity, sizeof( uint64_t ) );
	s->count = 0;
	for ( int i = 0; i < oldCap; ++i )
		if ( old[i] != 0 )
			gset_add( s, old[i] );
	free( old );
}

bool gset_add( gSet* s, uint64_t key )
{
	if ( 2 * ( s->count + 1 ) > s->capacity )
		gset_grow( s );
	uint64_t mask = (uint64_t)( s->capacity - 1 );
	uint64_t i = gset_hash( key ) & mask;
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

bool gset_contains( const gSet* s, uint64_t key )
{
	if ( s->capacity == 0 )
		return false;
	uint64_t mask = (uint64_t)( s->capacity - 1 );
	uint64_t i = gset_hash( key ) & mask;
	while ( s->keys[i] != 0 )
	{
		if ( s->keys[i] == key )
			return true;
		i = ( i + 1 ) & mask;
	}
	return false;
}

bool gset_remove( gSet* s, uint64_t key )
{
	if ( s->capacity == 0 )
		return false;
	uint64_t mask = (uint64_t)( s->capacity - 1 );
	uint64_t i = gset_hash( key ) & mask;
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
		gset_add( s, k );
		j = ( j + 1 ) & mask;
	}
	return true;
}

void gset_clear( gSet* s )
{
	if ( s->keys )
		memset( s->keys, 0, sizeof( uint64_t ) * (size_t)s->capacity );
	s->count = 0;
}

void gset_free( gSet* s )
{
	free( s->keys );
	memset( s, 0, sizeof( *s ) );
}

int gid_alloc( gIdPool* p )
{
	if ( p->freeIds.count > 0 )
	{
		p->freeIds.count -= 1;
		return p->freeIds.data[p->freeIds.count];
	}
	return p->next++;
}

void gid_free( gIdPool* p, int id )
{
	gia_push( &p->freeIds, id );
}

int gid_count( const gIdPool* p )
{
	return p->next - p->freeIds.count;
}

bool gbits_get( const gBits* b, int i )
{
	int w = i >> 6;
	if ( w >= b->wordCount )
		return false;
	return ( b->words[w] >> ( i & 63 ) ) & 1u;
}

void gbits_set( gBits* b, int i )
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

void gbits_clear( gBits* b, int i )
{
	int w = i >> 6;
	if ( w < b->wordCount )
		b->words[w] &= ~( (uint64_t)1 << ( i & 63 ) );
}

void gbits_free( gBits* b )
{
	free( b->words );
	memset( b, 0, sizeof( *b ) );
}
