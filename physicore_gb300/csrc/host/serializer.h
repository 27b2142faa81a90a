// serializer.h -- output of a microenvironment's state at a simulation time
// (reactions-diffusion/biofvm/include/biofvm/serializer.h).
#pragma once

#include "types.h"

namespace physicore::biofvm {

struct microenvironment;

class serializer
{
public:
	virtual void serialize(const microenvironment& m, real_t current_time) = 0;
	virtual ~serializer() = default;
};

} // namespace physicore::biofvm
