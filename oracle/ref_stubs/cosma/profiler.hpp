// Stand-in for the reference's profiler: the region markers compile to nothing.
#pragma once
#define PE(name)
#define PL()
