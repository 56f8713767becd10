// Stand-in: the functions the reference uses live in glm.hpp of this shim.
#pragma once
