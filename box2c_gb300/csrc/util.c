/*
 * util.c -- host containers of the step driver.
 *
 * Restates the semantics the step path depends on: swap-remove arrays (reference
 * src/block_array.c), the LIFO id pool (src/id_pool.c:21-45), bit sets (src/bitset.c)
 * and a membership-only hash set (src/table.c).
 */
#include "host.h"

#include <stdatomic.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------ host memory
 * Reference src/allocate.c:39-107.  Every host block of the library comes from the
 * allocator a caller installs with b2SetAllocator (requests are multiples of 32 bytes,
 * alignment 32), else from aligned_alloc; b2GetByteCount reports the bytes in use.
 * Each block starts with a 32-byte header holding its size, so resizing and freeing
 * need no size from the caller.  Pinned mirrors of device arrays come from the CUDA
 * runtime (cudaHostAlloc) and are not counted.  A request the allocator refuses
 * returns null: the caller keeps its state, and the failure is counted so that the API
 * call in progress can mark its world failed (b2World_GetStatus) instead of crashing.
 * The allocator must not change while library blocks are live. */
#define B2G_ALIGN 32

static b2AllocFcn* s_allocFcn;
static b2FreeFcn* s_freeFcn;
static _Atomic long long s_byteCount;
static _Atomic int s_allocFailures;

void b2SetAllocator( b2AllocFcn* allocFcn, b2FreeFcn* freeFcn )
{
	s_allocFcn = allocFcn;
	s_freeFcn = freeFcn;
}

int b2GetByteCount( void ) { return (int)atomic_load_explicit( &s_byteCount, memory_order_relaxed ); }

int b2g_alloc_failures( void ) { return atomic_load_explicit( &s_allocFailures, memory_order_relaxed ); }

void b2g_note_alloc_failure( void ) { atomic_fetch_add_explicit( &s_allocFailures, 1, memory_order_relaxed ); }

void* b2g_alloc( size_t size )
{
	size_t total = ( ( size + B2G_ALIGN - 1 ) & ~(size_t)( B2G_ALIGN - 1 ) ) + B2G_ALIGN;
	void* block = NULL;
	if ( total <= 0xFFFFFFFFu )
		block = s_allocFcn ? s_allocFcn( (unsigned int)total, B2G_ALIGN ) : aligned_alloc( B2G_ALIGN, total );
	if ( block == NULL )
	{
		b2g_note_alloc_failure();
		return NULL;
	}
	*(size_t*)block = size;
	atomic_fetch_add_explicit( &s_byteCount, (long long)size, memory_order_relaxed );
	return (char*)block + B2G_ALIGN;
}

void* b2g_calloc( size_t count, size_t size )
{
	void* p = b2g_alloc( count * size );
	if ( p )
		memset( p, 0, count * size );
	return p;
}

void b2g_free( void* p )
{
	if ( p == NULL )
		return;
	char* block = (char*)p - B2G_ALIGN;
	atomic_fetch_sub_explicit( &s_byteCount, (long long)*(size_t*)block, memory_order_relaxed );
	if ( s_freeFcn )
		s_freeFcn( block );
	else
		free( block );
}

void* b2g_realloc( void* p, size_t size )
{
	if ( p == NULL )
		return b2g_alloc( size );
	size_t old = *(size_t*)( (char*)p - B2G_ALIGN );
	void* q = b2g_alloc( size );
	if ( q == NULL )
		return NULL;
	memcpy( q, p, old < size ? old : size );
	b2g_free( p );
	return q;
}

bool gia_reserve( gIntArray* a, int count )
{
	if ( count <= a->capacity )
		return true;
	int cap = a->capacity < 16 ? 16 : 2 * a->capacity;
	while ( cap < count )
		cap *= 2;
	int* d = (int*)b2g_realloc( a->data, sizeof( int ) * (size_t)cap );
	if ( d == NULL )
		return false;
	a->data = d;
	a->capacity = cap;
	return true;
}

void gia_push( gIntArray* a, int v )
{
	if ( a->count == a->capacity && gia_reserve( a, a->count + 1 ) == false )
		return;
	a->data[a->count++] = v;
}

int gia_remove_swap( gIntArray* a, int index )
{
	/* an index an out-of-memory push never stored is ignored */
	if ( index < 0 || index >= a->count )
		return -1;
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
	b2g_free( a->data );
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

static bool gset_grow( gSet* s )
{
	int oldCap = s->capacity;
	uint64_t* old = s->keys;
	int cap = oldCap == 0 ? 64 : 2 * oldCap;
	uint64_t* keys = (uint64_t*)b2g_calloc( (size_t)cap, sizeof( uint64_t ) );
	if ( keys == NULL )
		return false;
	s->capacity = cap;
	s->keys = keys;
	s->count = 0;
	for ( int i = 0; i < oldCap; ++i )
		if ( old[i] != 0 )
			gset_add( s, old[i] );
	b2g_free( old );
	return true;
}

bool gset_add( gSet* s, uint64_t key )
{
	/* with no room to grow the key is reported present, never written past the table */
	if ( 2 * ( s->count + 1 ) > s->capacity && gset_grow( s ) == false && s->count + 1 >= s->capacity )
		return true;
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
	b2g_free( s->keys );
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

void gid_unalloc( gIdPool* p, int id )
{
	if ( id == p->next - 1 )
		p->next -= 1;
	else
		gia_push( &p->freeIds, id );
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
		uint64_t* words = (uint64_t*)b2g_realloc( b->words, sizeof( uint64_t ) * (size_t)n );
		if ( words == NULL )
			return;
		b->words = words;
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
	b2g_free( b->words );
	memset( b, 0, sizeof( *b ) );
}
