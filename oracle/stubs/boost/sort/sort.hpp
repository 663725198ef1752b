/* include/physics/boundary.h includes this header but calls nothing from
 * it on the path the oracle compiles.  Oracle build only. */
#pragma once
