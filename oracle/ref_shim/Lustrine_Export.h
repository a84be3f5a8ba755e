/* Stand-in for the CMake-generated export header the reference's sources
 * include (CMakeLists.txt:116-122): symbols stay at default visibility. */
#pragma once
#define LUSTRINE_EXPORT
