// Forwarding header: the reference includes "./include/glm/glm.hpp".
#include "../../glm/glm.hpp"
