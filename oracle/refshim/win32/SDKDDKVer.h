#pragma once
/* Empty stand-in for an MSVC/Windows SDK header: the reference includes it but
   uses nothing from it on the paths compiled here. */
