/* Empty stand-in for SDL's SDL_rect.h. The simulation header of the
 * reference includes it but uses nothing from it. Test infrastructure only. */
#pragma once
