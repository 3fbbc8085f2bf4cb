"""The reference's own benchmark scenes and world tests compile against include/ and link
against libbox2d_gb300.so with no missing symbol (a caller swaps the library in
unchanged).  Link only: running them needs a GPU.  Skipped where the reference sources
are absent."""
import os
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = "/root/reference"

STUB = r"""
#include "box2d/box2d.h"
b2WorldId JointGrid( b2WorldDef* def );
b2WorldId LargePyramid( b2WorldDef* def );
b2WorldId ManyPyramids( b2WorldDef* def );
b2WorldId Smash( b2WorldDef* def );
b2WorldId Tumbler( b2WorldDef* def );
int WorldTest( void );
int main( int argc, char** argv )
{
	(void)argv;
	if ( argc < 100 )
		return 0;
	b2WorldDef def = b2DefaultWorldDef();
	JointGrid( &def );
	LargePyramid( &def );
	ManyPyramids( &def );
	Smash( &def );
	Tumbler( &def );
	return WorldTest();
}
"""


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "benchmark")), reason="reference sources not present")
def test_reference_benchmarks_and_world_test_link(tmp_path):
    import box2c_gb300
    lib = box2c_gb300.build()
    stub = tmp_path / "main.c"
    stub.write_text(STUB)
    sources = [os.path.join(REF, "benchmark", f) for f in
               ("joint_grid.c", "large_pyramid.c", "many_pyramids.c", "smash.c", "tumbler.c")]
    sources.append(os.path.join(REF, "test", "test_world.c"))
    exe = str(tmp_path / "linked")
    r = subprocess.run(["gcc", "-std=gnu17", "-O1", "-I", os.path.join(REPO, "include"), "-I", os.path.join(REF, "test"),
                        str(stub), *sources, "-L", os.path.dirname(lib), "-lbox2d_gb300",
                        "-Wl,-rpath," + os.path.dirname(lib), "-lm", "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
