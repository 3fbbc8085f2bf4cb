/*
 * tree_check.c -- the library's host dynamic tree (box2c_gb300/csrc/tree.c) against the
 * oracle's (oracle/b2o_tree.c, pinned to the reference): the same seeded sequence of
 * proxy creates, moves, enlargements, destroys and partial rebuilds must leave both trees
 * with the same root, node count and every node slot (box bits, links, height), and
 * every query must report the same leaves in the same order (the order fixes contact
 * ids).  Prints "ok" and exits 0, or the first difference and exits 1.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

void* pt_new( void );
void pt_free( void* t );
int pt_create( void* t, const float* b, int user );
void pt_destroy( void* t, int id );
void pt_move( void* t, int id, const float* b );
void pt_enlarge( void* t, int id, const float* b );
void pt_rebuild( void* t );
int pt_query( void* t, const float* b, int* out, int cap );
int pt_dump( void* t, int* out, int cap );

void* ot_new( void );
void ot_free( void* t );
int ot_create( void* t, const float* b, int user );
void ot_destroy( void* t, int id );
void ot_move( void* t, int id, const float* b );
void ot_enlarge( void* t, int id, const float* b );
void ot_rebuild( void* t );
int ot_query( void* t, const float* b, int* out, int cap );
int ot_dump( void* t, int* out, int cap );

#define MAXP 4096
#define CAP ( 1 << 20 )

static unsigned long long s_state = 0x9E3779B97F4A7C15ull;
static float uniform( float lo, float hi )
{
	s_state = s_state * 6364136223846793005ull + 1442695040888963407ull;
	return lo + ( hi - lo ) * (float)( ( s_state >> 40 ) & 0xFFFFFF ) / 16777216.0f;
}
static int pick( int n ) { return (int)uniform( 0.0f, (float)n ) % n; }

static void random_box( float* b )
{
	float x = uniform( 0.0f, 100.0f ), y = uniform( 0.0f, 100.0f );
	float hx = uniform( 0.2f, 2.0f ), hy = uniform( 0.2f, 2.0f );
	b[0] = x - hx;
	b[1] = y - hy;
	b[2] = x + hx;
	b[3] = y + hy;
}

static int s_a[CAP], s_b[CAP];

static int compare( void* p, void* o, const char* when, int round )
{
	int na = pt_dump( p, s_a, CAP ), nb = ot_dump( o, s_b, CAP );
	if ( na != nb || memcmp( s_a, s_b, sizeof( int ) * (size_t)( na < CAP ? na : CAP ) ) != 0 )
	{
		printf( "trees differ after %s in round %d\n", when, round );
		return 1;
	}
	for ( int q = 0; q < 20; ++q )
	{
		float box[4];
		random_box( box );
		box[0] -= 3.0f;
		box[1] -= 3.0f;
		box[2] += 3.0f;
		box[3] += 3.0f;
		na = pt_query( p, box, s_a, CAP );
		nb = ot_query( o, box, s_b, CAP );
		if ( na != nb || memcmp( s_a, s_b, sizeof( int ) * (size_t)na ) != 0 )
		{
			printf( "queries differ after %s in round %d\n", when, round );
			return 1;
		}
	}
	return 0;
}

int main( void )
{
	void* p = pt_new();
	void* o = ot_new();
	static float boxes[MAXP][4];
	static int idP[MAXP], idO[MAXP], live[MAXP];
	int count = 0;
	for ( ; count < 300; ++count )
	{
		random_box( boxes[count] );
		idP[count] = pt_create( p, boxes[count], count );
		idO[count] = ot_create( o, boxes[count], count );
		live[count] = 1;
		if ( idP[count] != idO[count] )
			return printf( "proxy ids differ at create %d\n", count ), 1;
	}
	if ( compare( p, o, "creation", 0 ) )
		return 1;
	for ( int round = 1; round <= 40; ++round )
	{
		for ( int k = 0; k < 30; ++k )
		{
			int i = pick( count );
			if ( live[i] == 0 )
				continue;
			random_box( boxes[i] );
			pt_move( p, idP[i], boxes[i] );
			ot_move( o, idO[i], boxes[i] );
		}
		if ( compare( p, o, "moves", round ) )
			return 1;
		for ( int k = 0; k < 30; ++k )
		{
			int i = pick( count );
			if ( live[i] == 0 )
				continue;
			float m = uniform( 0.05f, 1.0f );
			boxes[i][0] -= m;
			boxes[i][1] -= m;
			boxes[i][2] += m;
			boxes[i][3] += m;
			pt_enlarge( p, idP[i], boxes[i] );
			ot_enlarge( o, idO[i], boxes[i] );
		}
		if ( compare( p, o, "enlargements", round ) )
			return 1;
		for ( int k = 0; k < 10; ++k )
		{
			int i = pick( count );
			if ( live[i] == 0 )
				continue;
			pt_destroy( p, idP[i] );
			ot_destroy( o, idO[i] );
			live[i] = 0;
		}
		for ( int k = 0; k < 10 && count < MAXP; ++k, ++count )
		{
			random_box( boxes[count] );
			idP[count] = pt_create( p, boxes[count], count );
			idO[count] = ot_create( o, boxes[count], count );
			live[count] = 1;
			if ( idP[count] != idO[count] )
				return printf( "proxy ids differ at create %d\n", count ), 1;
		}
		if ( compare( p, o, "destroys and creates", round ) )
			return 1;
		if ( round % 4 == 0 )
		{
			pt_rebuild( p );
			ot_rebuild( o );
			if ( compare( p, o, "rebuild", round ) )
				return 1;
		}
	}
	pt_free( p );
	ot_free( o );
	printf( "ok\n" );
	return 0;
}
