// The reference's GATECOUNT cost model (include/gatecounters.hpp) is not part
// of this engine; builds without -DGATECOUNT (the default) compile its hooks away.
#pragma once
#ifdef GATECOUNT
#error "GATECOUNT gate-cost tables are not provided by suqa_gb300 (use sq_get_stats for pass/gate counts)"
#endif
