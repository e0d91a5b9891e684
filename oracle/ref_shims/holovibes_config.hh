// Stand-in for Backend/includes/core/holovibes_config.hh in the comparison build: the Windows
// executable-directory helpers are not needed by the compute translation units.
#pragma once
