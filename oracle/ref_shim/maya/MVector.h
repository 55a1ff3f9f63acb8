/* Minimal stand-in for the Maya type named by util/math.h (test shim only). */
#pragma once
class MVector { public: double x, y, z; };
