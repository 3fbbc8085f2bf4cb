/*
 * pool_check.c -- host check of the fork-join pool (box2c_gb300/csrc/pool.c): every
 * index of a job is visited exactly once, gpool_try_for declines while another thread's
 * job runs and when called from inside a job, and both run again afterwards.
 * Prints "ok" and exits 0, or names the failed check and exits 1.
 */
#include "host.h"

#include <pthread.h>
#include <stdatomic.h>
#include <stdio.h>
#include <string.h>
#include <unistd.h>

#define N 100000

static atomic_int s_hits[N];
static atomic_int s_nestedRan, s_nestedDeclined;
static atomic_int s_inside, s_release;

static void count_range( int begin, int end, void* ctx )
{
	(void)ctx;
	for ( int i = begin; i < end; ++i )
		atomic_fetch_add( &s_hits[i], 1 );
}

static void nested_range( int begin, int end, void* ctx )
{
	(void)ctx;
	(void)begin;
	(void)end;
	if ( gpool_try_for( 1000, 10, count_range, NULL ) )
		atomic_fetch_add( &s_nestedRan, 1 );
	else
		atomic_fetch_add( &s_nestedDeclined, 1 );
}

/* holds the pool until released */
static void hold_range( int begin, int end, void* ctx )
{
	(void)ctx;
	(void)end;
	if ( begin == 0 )
	{
		atomic_store( &s_inside, 1 );
		while ( atomic_load( &s_release ) == 0 )
			usleep( 100 );
	}
}

static void* holder( void* arg )
{
	(void)arg;
	gpool_for( 64, 1, hold_range, NULL );
	return NULL;
}

static int fail( const char* what )
{
	printf( "failed: %s\n", what );
	return 1;
}

int main( void )
{
	if ( gpool_threads() < 2 )
	{
		printf( "ok (one thread: the pool runs every range on the caller)\n" );
		return 0;
	}
	gpool_for( N, 64, count_range, NULL );
	for ( int i = 0; i < N; ++i )
		if ( atomic_load( &s_hits[i] ) != 1 )
			return fail( "gpool_for visits every index once" );

	gpool_for( 256, 1, nested_range, NULL );
	if ( atomic_load( &s_nestedRan ) != 0 || atomic_load( &s_nestedDeclined ) != 256 )
		return fail( "gpool_try_for declines inside a job" );

	pthread_t t;
	pthread_create( &t, NULL, holder, NULL );
	while ( atomic_load( &s_inside ) == 0 )
		usleep( 100 );
	memset( s_hits, 0, sizeof( s_hits ) );
	bool ran = gpool_try_for( N, 64, count_range, NULL );
	atomic_store( &s_release, 1 );
	pthread_join( t, NULL );
	if ( ran )
		return fail( "gpool_try_for declines while another thread's job runs" );

	if ( gpool_try_for( N, 64, count_range, NULL ) == false )
		return fail( "gpool_try_for runs when the pool is free" );
	for ( int i = 0; i < N; ++i )
		if ( atomic_load( &s_hits[i] ) != 1 )
			return fail( "gpool_try_for visits every index once" );
	printf( "ok\n" );
	return 0;
}
