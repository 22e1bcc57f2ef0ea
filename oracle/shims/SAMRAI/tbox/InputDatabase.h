/* Empty stand-in: the solver headers include this but the serial path uses nothing from it. */
#pragma once
