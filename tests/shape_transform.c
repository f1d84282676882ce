/* Test-only transform function for the shape tests (compiled by tests/shape_util.py): the same formula
 * as the one the reference goldens were made with (tests/golden/make_shape_golden.py). */
#include "DoonEngine/voxelShapes.h"
#include <math.h>

DNvoxel dn_test_shape_transform(DNvec3 pos, DNvec3 normal, DNvoxel vox, DNvec3 mn, DNvec3 mx, DNmat4 inv, void* user)
{
	(void)user;
	const float lx = inv.m[0][0] * pos.x + inv.m[1][0] * pos.y + inv.m[2][0] * pos.z + inv.m[3][0] * 1.0f;
	const float ly = inv.m[0][1] * pos.x + inv.m[1][1] * pos.y + inv.m[2][1] * pos.z + inv.m[3][1] * 1.0f;
	vox.normal = normal;
	vox.albedo.r = (uint8_t)((int)floorf(lx * 8.0f) & 255);
	vox.albedo.g = (uint8_t)((int)floorf(ly * 8.0f) & 255);
	vox.albedo.b = (uint8_t)((int)floorf((pos.z - mn.z) * 4.0f + mx.x) & 255);
	vox.material = normal.y > 0.0f ? 3 : 4;
	return vox;
}
