/*
 * Unit checks of the adjoint's row VJPs (warm start, solve, relax, restitution) and of
 * the position-integration and finalisation VJPs against central differences of the
 * forward routines they differentiate, at random inputs.  Built and run by
 * tests/test_gpu_adjoint_units.py; prints MISMATCH lines on failure.
 */
#include "adjoint.cu"
#include <stdio.h>

__device__ float frand( unsigned& s ) { s = s * 1664525u + 1013904223u; return ( ( s >> 8 ) & 0xFFFF ) / 65536.0f * 2.0f - 1.0f; }

struct SolveIn { Row r; DevState a, b; };
// objective: weighted sum of outputs (velocities and impulses)
__device__ float solve_obj( SolveIn x, int phase, const b2gStepConst& sc, const float* w )
{
	Row r = x.r; DevState a = x.a, b = x.b;
	if ( phase == 0 ) warm_lane( r, a, b );
	else if ( phase == 3 ) restitution_lane( r, a, b, sc.restitutionThreshold );
	else solve_lane( r, a, b, phase == 1, sc.inv_h, sc.pushout );
	return w[0] * a.v.x + w[1] * a.v.y + w[2] * a.w + w[3] * b.v.x + w[4] * b.v.y + w[5] * b.w + w[6] * r.ni[0] + w[7] * r.ni[1] +
		   w[8] * r.ti[0] + w[9] * r.ti[1];
}
__device__ float* slot( SolveIn& x, int i )
{
	float* F[] = { &x.a.v.x, &x.a.v.y, &x.a.w, &x.b.v.x, &x.b.v.y, &x.b.w, &x.r.ni[0], &x.r.ni[1], &x.r.ti[0], &x.r.ti[1],
				   &x.a.dp.x, &x.a.dp.y, &x.a.dq.c, &x.a.dq.s, &x.b.dp.x, &x.b.dp.y, &x.b.dq.c, &x.b.dq.s, &x.r.base[0], &x.r.base[1],
				   &x.r.nMass[0], &x.r.nMass[1], &x.r.tMass[0], &x.r.tMass[1], &x.r.n.x, &x.r.n.y, &x.r.rA[0].x, &x.r.rA[0].y,
				   &x.r.rB[0].x, &x.r.rB[0].y, &x.r.rA[1].x, &x.r.rA[1].y, &x.r.rB[1].x, &x.r.rB[1].y, &x.r.friction, &x.r.relVel[0], &x.r.relVel[1] };
	return F[i];
}
__global__ void k_check( int phase, unsigned seed )
{
	unsigned s = seed;
	b2gStepConst sc;
	memset( &sc, 0, sizeof( sc ) );
	sc.h = 1.0f / 240.0f; sc.inv_h = 240.0f; sc.inv_dt = 60.0f; sc.pushout = 3.0f; sc.restitutionThreshold = 1.0f;
	SolveIn x;
	memset( &x, 0, sizeof( x ) );
	Row& r = x.r;
	float ang = 0.3f * frand( s );
	r.n = gv( sinf( ang ), cosf( ang ) );
	r.friction = 0.6f; r.restitution = 0.3f;
	r.biasRate = 20.0f; r.massScale = 0.9f; r.impulseScale = 0.1f;
	r.mA = 1.0f; r.iA = 6.0f; r.mB = 0.7f; r.iB = 4.0f;
	r.count = 2;
	for ( int j = 0; j < 2; ++j )
	{
		r.rA[j] = gv( 0.5f * frand( s ), 0.5f * frand( s ) );
		r.rB[j] = gv( 0.5f * frand( s ), 0.5f * frand( s ) );
		r.base[j] = 0.01f * frand( s ) - ( j == 0 ? 0.005f : -0.004f );
		r.nMass[j] = 0.5f + 0.1f * frand( s );
		r.tMass[j] = 0.4f + 0.1f * frand( s );
		r.relVel[j] = -2.0f + 0.5f * frand( s );
		r.ni[j] = 0.3f + 0.1f * frand( s );
		r.ti[j] = 0.05f * frand( s );
		r.maxNi[j] = 0.2f;
	}
	x.a.v = gv( frand( s ), frand( s ) ); x.a.w = frand( s );
	x.b.v = gv( frand( s ), frand( s ) ); x.b.w = frand( s );
	x.a.dp = gv( 0.001f * frand( s ), 0.001f * frand( s ) ); x.a.dq = grot( 1.0f, 0.0f );
	x.b.dp = gv( 0.001f * frand( s ), 0.001f * frand( s ) ); x.b.dq = gnormrot( grot( 1.0f, 0.01f * frand( s ) ) );
	float w[10];
	for ( int i = 0; i < 10; ++i ) w[i] = frand( s );
	// adjoint
	BodyV aA = { w[0], w[1], w[2] }, aB = { w[3], w[4], w[5] };
	RowAdj ra;
	memset( &ra, 0, sizeof( ra ) );
	ra.ni[0] = w[6]; ra.ni[1] = w[7]; ra.ti[0] = w[8]; ra.ti[1] = w[9];
	float dpA[2] = { 0, 0 }, dqA[2] = { 0, 0 }, dpB[2] = { 0, 0 }, dqB[2] = { 0, 0 };
	if ( phase == 0 ) warm_vjp( r, aA, aB, ra );
	else if ( phase == 3 ) restitution_vjp( r, x.a, x.b, sc, aA, aB, ra );
	else solve_vjp( r, x.a, x.b, phase == 1, sc, aA, aB, ra, dpA, dqA, dpB, dqB );
	float adj[37] = { aA.vx, aA.vy, aA.w, aB.vx, aB.vy, aB.w, ra.ni[0], ra.ni[1], ra.ti[0], ra.ti[1], dpA[0], dpA[1], dqA[0], dqA[1],
					  dpB[0], dpB[1], dqB[0], dqB[1], ra.base[0], ra.base[1], ra.nMass[0], ra.nMass[1], ra.tMass[0], ra.tMass[1],
					  ra.n[0], ra.n[1], ra.rA[0][0], ra.rA[0][1], ra.rB[0][0], ra.rB[0][1], ra.rA[1][0], ra.rA[1][1], ra.rB[1][0],
					  ra.rB[1][1], ra.mu, ra.relVel[0], ra.relVel[1] };
	const char* names[37] = { "a.vx", "a.vy", "a.w", "b.vx", "b.vy", "b.w", "ni0", "ni1", "ti0", "ti1", "dpA.x", "dpA.y", "dqA.c", "dqA.s",
							  "dpB.x", "dpB.y", "dqB.c", "dqB.s", "base0", "base1", "nMass0", "nMass1", "tMass0", "tMass1", "n.x", "n.y",
							  "rA0.x", "rA0.y", "rB0.x", "rB0.y", "rA1.x", "rA1.y", "rB1.x", "rB1.y", "mu", "relVel0", "relVel1" };
	float eps = 1e-3f;
	for ( int i = 0; i < 37; ++i )
	{
		SolveIn p = x, m = x;
		*slot( p, i ) += eps;
		*slot( m, i ) -= eps;
		float fd = ( solve_obj( p, phase, sc, w ) - solve_obj( m, phase, sc, w ) ) / ( 2.0f * eps );
		float err = fabsf( fd - adj[i] );
		if ( err > 2e-3f * fmaxf( 1.0f, fabsf( fd ) ) )
			printf( "phase %d seed %u %-8s adj % .6f fd % .6f  MISMATCH\n", phase, seed, names[i], adj[i], fd );
	}
	printf( "phase %d seed %u done\n", phase, seed );
}

// body VJPs
__global__ void k_check_body( unsigned seed )
{
	unsigned s = seed;
	b2gStepConst sc;
	memset( &sc, 0, sizeof( sc ) );
	sc.h = 1.0f / 240.0f; sc.inv_dt = 60.0f;
	float pre[8] = { frand( s ), frand( s ), 3.0f * frand( s ), 0, 0.01f * frand( s ), 0.01f * frand( s ), 0, 0 };
	b2gRot dq = gnormrot( grot( 1.0f, 0.05f * frand( s ) ) );
	pre[6] = dq.c; pre[7] = dq.s;
	float w[11];
	for ( int i = 0; i < 11; ++i ) w[i] = frand( s );
	// IP: outputs v(2) w dp(2) dq(2)
	auto ip = [&]( const float* x ) {
		DevState st = state_of( make_float4( x[0], x[1], x[2], 0 ), make_float4( x[4], x[5], x[6], x[7] ) );
		integrate_position( st, sc.h );
		return w[4] * st.v.x + w[5] * st.v.y + w[6] * st.w + w[7] * st.dp.x + w[8] * st.dp.y + w[9] * st.dq.c + w[10] * st.dq.s;
	};
	float g[12] = { 0, 0, 0, 0, w[4], w[5], w[6], w[7], w[8], w[9], w[10], 0 };
	ip_vjp( pre, sc.h, g );
	int map[7] = { 0, 1, 2, 4, 5, 6, 7 };
	int gi[7] = { 4, 5, 6, 7, 8, 9, 10 };
	for ( int i = 0; i < 7; ++i )
	{
		float p[8], m[8];
		for ( int k = 0; k < 8; ++k ) p[k] = m[k] = pre[k];
		p[map[i]] += 1e-3f; m[map[i]] -= 1e-3f;
		float fd = ( ip( p ) - ip( m ) ) / 2e-3f;
		if ( fabsf( fd - g[gi[i]] ) > 2e-3f * fmaxf( 1.0f, fabsf( fd ) ) ) printf( "IP %d adj %f fd %f MISMATCH\n", i, g[gi[i]], fd );
	}
	// finalize: inputs q(2) dq(2) c(2) dp(2) -> outputs c'(2) q'(2)
	float qc = 0.8f, qs = 0.6f;
	auto fin = [&]( float a, float b, float c, float d, float dpx, float dpy ) {
		b2gRot q = gnormrot( gmulrot( grot( c, d ), grot( a, b ) ) );
		return w[0] * dpx + w[1] * dpy + w[2] * q.c + w[3] * q.s;
	};
	float gf[12] = { w[0], w[1], w[2], w[3], 0, 0, 0, 0, 0, 0, 0, 0 };
	finalize_vjp( qc, qs, dq.c, dq.s, gf );
	float in[6] = { qc, qs, dq.c, dq.s, 0, 0 };
	int gidx[6] = { 2, 3, 9, 10, 7, 8 };
	for ( int i = 0; i < 6; ++i )
	{
		float p[6], m[6];
		for ( int k = 0; k < 6; ++k ) p[k] = m[k] = in[k];
		p[i] += 1e-3f; m[i] -= 1e-3f;
		float fd = ( fin( p[0], p[1], p[2], p[3], p[4], p[5] ) - fin( m[0], m[1], m[2], m[3], m[4], m[5] ) ) / 2e-3f;
		if ( fabsf( fd - gf[gidx[i]] ) > 2e-3f * fmaxf( 1.0f, fabsf( fd ) ) ) printf( "FIN %d adj %f fd %f MISMATCH\n", i, gf[gidx[i]], fd );
	}
	printf( "body seed %u done\n", seed );
}

int main()
{
	for ( unsigned seed = 1; seed <= 6; ++seed )
	{
		for ( int ph = 0; ph < 4; ++ph )
			k_check<<<1, 1>>>( ph, seed );
		k_check_body<<<1, 1>>>( seed );
	}
	cudaError_t e = cudaDeviceSynchronize();
	printf( "status %s\n", cudaGetErrorString( e ) );
	return e == cudaSuccess ? 0 : 1;
}
