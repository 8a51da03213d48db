/* Stand-in (TEST INFRASTRUCTURE ONLY): the reference sources include this header but use
 * nothing from it beyond sundials_core.hpp. */
#pragma once
#include <sundials/sundials_core.hpp>
