// Stand-in for the absent OptiX SDK header (function-table stubs): empty.
#pragma once
