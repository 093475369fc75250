// The reference includes <glm/gtx/transform.hpp>; nothing from it is used on the solver path.
#include "../glm.hpp"
