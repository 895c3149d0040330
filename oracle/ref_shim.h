/*
 * Forced-include shim for compiling two reference headers in place
 * (tools/Rng.h and core/CDF.h of RaytracerNew2/src).  Both only need the
 * scalar type `real` from core/Geometry.h, which itself pulls in Eigen (not
 * installed here).  Defining Geometry.h's include guard and `real` lets the
 * reference's own code compile unchanged.  TEST INFRASTRUCTURE ONLY.
 */
#ifndef RT_REF_SHIM_H
#define RT_REF_SHIM_H
#define H__GEOMETRY_160520150025__H 1
#include <cmath>
#include <cstdint>
#include <vector>
#include <algorithm>
namespace priv { typedef float real; }
using priv::real;
#endif
