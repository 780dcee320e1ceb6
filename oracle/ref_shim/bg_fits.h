// Stand-in: the reference includes this header but the code compiled here uses nothing from it.
#pragma once
