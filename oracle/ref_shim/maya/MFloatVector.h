/* Minimal stand-in for the Maya type named by util/math.h (test shim only). */
#pragma once
class MFloatVector { public: float x, y, z; };
