// Oracle-only stub: the wrappers declare Boost serialization hooks that the oracle never calls.
#pragma once
namespace boost { namespace serialization { class access {}; } }
