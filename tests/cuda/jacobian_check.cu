/*
 * Unit checks of the adjoint's row-preparation VJP and of the dual-number manifold
 * Jacobian against central differences of the float routines they differentiate.
 * Built and run by tests/test_gpu_adjoint_units.py; prints MISMATCH lines on failure.
 */
#include "adjoint.cu"
#include <stdio.h>
__device__ float frand( unsigned& s ) { s = s * 1664525u + 1013904223u; return ( ( s >> 8 ) & 0xFFFF ) / 65536.0f * 2.0f - 1.0f; }

// prepare: inputs manifold (n, anchors, sep) + velocities; outputs Row fields
struct PIn { b2gManifold m; DevState a, b; };
__device__ float prep_obj( PIn x, const float* w, float4 mA, float4 mB, const float* soft )
{
	Row r;
	prepare_row( r, &x.m, 0, 1, mA, mB, x.a, x.b, 0.6f, 0.0f, soft, 1.0f );
	float o = 0.0f;
	int k = 0;
	o += w[k++] * r.n.x; o += w[k++] * r.n.y;
	for ( int j = 0; j < 2; ++j )
	{
		o += w[k++] * r.rA[j].x; o += w[k++] * r.rA[j].y; o += w[k++] * r.rB[j].x; o += w[k++] * r.rB[j].y;
		o += w[k++] * r.base[j]; o += w[k++] * r.nMass[j]; o += w[k++] * r.tMass[j]; o += w[k++] * r.relVel[j];
		o += w[k++] * r.ni[j]; o += w[k++] * r.ti[j];
	}
	return o;
}
__global__ void k_prep( unsigned seed )
{
	unsigned s = seed;
	PIn x;
	memset( &x, 0, sizeof( x ) );
	float ang = 0.4f * frand( s );
	x.m.normal = gv( sinf( ang ), cosf( ang ) );
	x.m.count = 2;
	for ( int j = 0; j < 2; ++j )
	{
		x.m.pts[j].anchorA = gv( 0.5f * frand( s ), 0.5f * frand( s ) );
		x.m.pts[j].anchorB = gv( 0.5f * frand( s ), 0.5f * frand( s ) );
		x.m.pts[j].separation = 0.01f * frand( s );
		x.m.pts[j].normalImpulse = 0.3f;
		x.m.pts[j].tangentImpulse = 0.1f;
	}
	x.a.v = gv( frand( s ), frand( s ) ); x.a.w = frand( s ); x.a.dq = grot( 1, 0 );
	x.b.v = gv( frand( s ), frand( s ) ); x.b.w = frand( s ); x.b.dq = grot( 1, 0 );
	float4 mA = make_float4( 1.0f, 1.0f, 0.16f, 6.0f ), mB = make_float4( 1.4f, 0.7f, 0.25f, 4.0f );
	float soft[3] = { 20.0f, 0.9f, 0.1f };
	float w[22];
	for ( int i = 0; i < 22; ++i ) w[i] = frand( s );
	Row r;
	prepare_row( r, &x.m, 0, 1, mA, mB, x.a, x.b, 0.6f, 0.0f, soft, 1.0f );
	RowAdj ra;
	memset( &ra, 0, sizeof( ra ) );
	int k = 0;
	ra.n[0] = w[k++]; ra.n[1] = w[k++];
	for ( int j = 0; j < 2; ++j )
	{
		ra.rA[j][0] = w[k++]; ra.rA[j][1] = w[k++]; ra.rB[j][0] = w[k++]; ra.rB[j][1] = w[k++];
		ra.base[j] = w[k++]; ra.nMass[j] = w[k++]; ra.tMass[j] = w[k++]; ra.relVel[j] = w[k++];
		ra.ni[j] = w[k++]; ra.ti[j] = w[k++];
	}
	float mAdj[12], lam[4];
	BodyV aA = { 0, 0, 0 }, aB = { 0, 0, 0 };
	prepare_vjp( r, x.a, x.b, ra, 1.0f, mAdj, aA, aB, lam );
	float* F[19] = { &x.m.normal.x, &x.m.normal.y, &x.m.pts[0].anchorA.x, &x.m.pts[0].anchorA.y, &x.m.pts[0].anchorB.x,
					 &x.m.pts[0].anchorB.y, &x.m.pts[0].separation, &x.m.pts[1].anchorA.x, &x.m.pts[1].anchorA.y,
					 &x.m.pts[1].anchorB.x, &x.m.pts[1].anchorB.y, &x.m.pts[1].separation, &x.a.v.x, &x.a.v.y, &x.a.w, &x.b.v.x,
					 &x.b.v.y, &x.b.w, &x.m.pts[0].normalImpulse };
	float adj[19] = { mAdj[0], mAdj[1], mAdj[2], mAdj[3], mAdj[4], mAdj[5], mAdj[6], mAdj[7], mAdj[8], mAdj[9], mAdj[10], mAdj[11],
					  aA.vx, aA.vy, aA.w, aB.vx, aB.vy, aB.w, lam[0] };
	for ( int i = 0; i < 19; ++i )
	{
		PIn p = x, m = x;
		float* fp = (float*)( (char*)&p + ( (char*)F[i] - (char*)&x ) );
		float* fm = (float*)( (char*)&m + ( (char*)F[i] - (char*)&x ) );
		*fp += 1e-3f; *fm -= 1e-3f;
		float fd = ( prep_obj( p, w, mA, mB, soft ) - prep_obj( m, w, mA, mB, soft ) ) / 2e-3f;
		if ( fabsf( fd - adj[i] ) > 2e-3f * fmaxf( 1.0f, fabsf( fd ) ) ) printf( "PREP seed %u in %d adj %f fd %f MISMATCH\n", seed, i, adj[i], fd );
	}
	printf( "prep seed %u done\n", seed );
}

// manifold Jacobian vs FD of the float narrowphase (anchors shifted to centres)
__device__ void float_manifold( const b2gShapeGeo& gA, const b2gShapeGeo& gB, const float* sa, const float* sb, float* out, int* ids )
{
	b2gXf xa, xb;
	xa.q = grot( sa[2], sa[3] ); xa.p = gsub( gv( sa[0], sa[1] ), grotate( xa.q, gv( sa[4], sa[5] ) ) );
	xb.q = grot( sb[2], sb[3] ); xb.p = gsub( gv( sb[0], sb[1] ), grotate( xb.q, gv( sb[4], sb[5] ) ) );
	b2gManifold m;
	gcollide_shapes( &m, &gA, xa, &gB, xb, nullptr );
	b2gVec offA = grotate( xa.q, gv( sa[4], sa[5] ) ), offB = grotate( xb.q, gv( sb[4], sb[5] ) );
	for ( int i = 0; i < 12; ++i ) out[i] = 0;
	out[0] = m.normal.x; out[1] = m.normal.y;
	for ( int j = 0; j < m.count; ++j )
	{
		b2gVec a = gsub( m.pts[j].anchorA, offA ), b = gsub( m.pts[j].anchorB, offB );
		out[2 + 5 * j] = a.x; out[3 + 5 * j] = a.y; out[4 + 5 * j] = b.x; out[5 + 5 * j] = b.y; out[6 + 5 * j] = m.pts[j].separation;
	}
	ids[0] = m.count;
	ids[1] = m.count > 0 ? m.pts[0].id : -1;
	ids[2] = m.count > 1 ? m.pts[1].id : -1;
}
__global__ void k_jac( unsigned seed, int scene )
{
	unsigned s = seed;
	b2gShapeGeo gA, gB;
	memset( &gA, 0, sizeof( gA ) ); memset( &gB, 0, sizeof( gB ) );
	auto box = [&]( b2gShapeGeo& g, float hx, float hy, float cx, float cy ) {
		g.type = 3; g.count = 4; g.radius = 0;
		g.v[0] = gv( cx - hx, cy - hy ); g.v[1] = gv( cx + hx, cy - hy ); g.v[2] = gv( cx + hx, cy + hy ); g.v[3] = gv( cx - hx, cy + hy );
		g.n[0] = gv( 0, -1 ); g.n[1] = gv( 1, 0 ); g.n[2] = gv( 0, 1 ); g.n[3] = gv( -1, 0 );
	};
	float sa[6], sb[6];
	if ( scene == 0 )
	{
		box( gA, 100.0f, 0.5f, 0.0f, 0.0f ); box( gB, 0.5f, 0.5f, 0, 0 );
		float t = 0.2f * frand( s );
		float sA_[6] = { 0.0f, -0.5f, 1.0f, 0.0f, 0, 0 };
		float sB_[6] = { 0.3f, 0.5f - 0.005f + 0.01f * frand( s ) + 0.5f * fabsf( sinf( t ) ), cosf( t ), sinf( t ), 0, 0 };
		for ( int i = 0; i < 6; ++i ) { sa[i] = sA_[i]; sb[i] = sB_[i]; }
	}
	else
	{
		box( gA, 0.5f, 0.5f, 0, 0 ); box( gB, 0.5f, 0.5f, 0, 0 );
		float t = 0.1f * frand( s ), u = 0.1f * frand( s );
		float sA_[6] = { 0.0f, 0.0f, cosf( t ), sinf( t ), 0, 0 };
		float sB_[6] = { 1.0f + 0.01f * frand( s ), 0.2f * frand( s ), cosf( u ), sinf( u ), 0, 0 };
		for ( int i = 0; i < 6; ++i ) { sa[i] = sA_[i]; sb[i] = sB_[i]; }
	}
	// start records for manifold_jacobian: c.x c.y q.c q.s lc.x lc.y p.x p.y
	float stA[12], stB[12];
	b2gXf xa, xb;
	xa.q = grot( sa[2], sa[3] ); xa.p = gsub( gv( sa[0], sa[1] ), grotate( xa.q, gv( sa[4], sa[5] ) ) );
	xb.q = grot( sb[2], sb[3] ); xb.p = gsub( gv( sb[0], sb[1] ), grotate( xb.q, gv( sb[4], sb[5] ) ) );
	float a8[8] = { sa[0], sa[1], sa[2], sa[3], sa[4], sa[5], xa.p.x, xa.p.y }, b8[8] = { sb[0], sb[1], sb[2], sb[3], sb[4], sb[5], xb.p.x, xb.p.y };
	for ( int i = 0; i < 8; ++i ) { stA[i] = a8[i]; stB[i] = b8[i]; }
	b2gManifold rec;
	gcollide_shapes( &rec, &gA, xa, &gB, xb, nullptr );
	b2gVec offA = grotate( xa.q, gv( sa[4], sa[5] ) ), offB = grotate( xb.q, gv( sb[4], sb[5] ) );
	for ( int j = 0; j < rec.count; ++j ) { rec.pts[j].anchorA = gsub( rec.pts[j].anchorA, offA ); rec.pts[j].anchorB = gsub( rec.pts[j].anchorB, offB ); }
	float jac[72];
	bool same = manifold_jacobian( gA, gB, stA, stB, scene == 1, true, rec, jac );
	if ( !same ) printf( "JAC scene %d seed %u replay mismatch (count %d)\n", scene, seed, rec.count );
	// FD over directions: c.x c.y angle for A (scene 1 only) and B
	for ( int d = 0; d < 6; ++d )
	{
		if ( scene == 0 && d < 3 ) continue;
		float pa[6], ma[6], pb[6], mb[6];
		for ( int i = 0; i < 6; ++i ) { pa[i] = ma[i] = sa[i]; pb[i] = mb[i] = sb[i]; }
		float e = 1e-3f;
		float* P = d < 3 ? pa : pb; float* M = d < 3 ? ma : mb;
		int k = d % 3;
		if ( k < 2 ) { P[k] += e; M[k] -= e; }
		else
		{
			float th = atan2f( P[3], P[2] );
			P[2] = cosf( th + e ); P[3] = sinf( th + e ); M[2] = cosf( th - e ); M[3] = sinf( th - e );
		}
		float op[12], om[12];
		int ip[3], im[3];
		float_manifold( gA, gB, pa, pb, op, ip );
		float_manifold( gA, gB, ma, mb, om, im );
		/* a step that switches the reference face or the clipped features crosses a
		 * discontinuity of the manifold: no derivative to compare there */
		int i0[3] = { rec.count, rec.count > 0 ? rec.pts[0].id : -1, rec.count > 1 ? rec.pts[1].id : -1 };
		bool smooth = true;
		for ( int i = 0; i < 3; ++i )
			smooth = smooth && ip[i] == i0[i] && im[i] == i0[i];
		if ( !smooth )
			continue;
		float o0[12];
		int i0_[3];
		float_manifold( gA, gB, sa, sb, o0, i0_ );
		for ( int o = 0; o < 12; ++o )
		{
			float fd = ( op[o] - om[o] ) / ( 2 * e );
			/* one-sided differences that disagree: the step crosses a kink (e.g. the
			 * reference face switching between two nearly parallel faces) */
			float fplus = ( op[o] - o0[o] ) / e, fminus = ( o0[o] - om[o] ) / e;
			if ( fabsf( fplus - fminus ) > 1e-2f * fmaxf( 1.0f, fabsf( fd ) ) )
				continue;
			if ( fabsf( fd - jac[o * 6 + d] ) > 5e-3f * fmaxf( 1.0f, fabsf( fd ) ) )
				printf( "JAC scene %d seed %u out %d dir %d adj %f fd %f MISMATCH\n", scene, seed, o, d, jac[o * 6 + d], fd );
		}
	}
	printf( "jac scene %d seed %u done (count %d)\n", scene, seed, rec.count );
}
int main()
{
	for ( unsigned seed = 1; seed <= 5; ++seed )
	{
		k_prep<<<1, 1>>>( seed );
		k_jac<<<1, 1>>>( seed, 0 );
		k_jac<<<1, 1>>>( seed, 1 );
	}
	cudaError_t e = cudaDeviceSynchronize();
	printf( "status %s\n", cudaGetErrorString( e ) );
	return e == cudaSuccess ? 0 : 1;
}
