// included by the reference's network.h; nothing from it is used
#pragma once
