// Stand-in for serac's generated configuration header (no optional TPLs).
#pragma once
