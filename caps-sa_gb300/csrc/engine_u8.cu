// engine_u8.cu — suffix-sort engine instantiated for uint8_t symbols.
#include "engine_impl.cuh"

namespace capssa {
capssa_status engine_build_u8(Ctx &c, const EngineArgs &a) { return engine_build_t<uint8_t>(c, a); }
}  // namespace capssa
