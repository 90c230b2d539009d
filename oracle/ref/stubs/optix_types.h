/* Stand-in for the one OptiX type the reference's kd-tree code uses: an
 * axis-aligned box of six floats (OptixAabb in the OptiX 7 SDK). */
#pragma once
struct OptixAabb { float minX, minY, minZ, maxX, maxY, maxZ; };
