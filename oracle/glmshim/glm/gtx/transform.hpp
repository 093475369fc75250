// The reference includes <glm/gtx/transform.hpp>; translate and rotate (used
// by its Canvas2D voxeliser, not by the solver path) are in ../glm.hpp.
#include "../glm.hpp"
