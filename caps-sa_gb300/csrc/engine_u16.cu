// engine_u16.cu — suffix-sort engine instantiated for uint16_t symbols.
#include "engine_impl.cuh"

namespace capssa {
capssa_status engine_build_u16(Ctx &c, const EngineArgs &a) { return engine_build_t<uint16_t>(c, a); }
}  // namespace capssa
